// Split-precision FFT stages on the 5th-generation tensor cores (tcgen05).
//
// Same mathematics as split_tc.cu (radix-16 Stockham stages of N = 256 / 4096
// as Y = F16 X with BF16 limbs and FP32 accumulation; here three limbs of X
// are cut by truncation, so they represent X exactly), laid out for
// tcgen05.mma: per stage the 256 DFT columns of a CTA's 4096 points form the
// M dimension, so each product is
//   D[j][n] += sum_kk A[j][kk] B[n][kk],   M = 128 columns j, N = 32, K = 32,
// with A = the columns' inputs [Xr(0..15) | Xi(0..15)] (one BF16 limb) and
// B = the real form of F16^T (one limb): B[k][m] = Re F, B[k][16+m] = -Im F,
// B[16+k][m] = Im F, B[16+k][16+m] = Re F.  D (FP32, 32 TMEM columns per
// 128 DFT columns) holds Yr(0..15) | Yi(0..15) of column j in TMEM lane j.
//
// Per stage: every thread gathers its column (shared memory), applies the
// stage twiddle in FP32, splits into limbs and writes them as the A operand
// (canonical K-major layout without swizzle: 8-row x 16-byte core matrices,
// K-adjacent ones 128 B apart, 8-row groups 512 B apart); one thread issues
// the 2 tiles x products x 2 K-halves of MMAs and commits them to an
// mbarrier; after the wait every thread reads its D row with tcgen05.ld and
// scatters the 16 outputs to their Stockham positions.  Persistent CTAs (two
// per SM) allocate 64 TMEM columns once.  Waits are bounded: on timeout the
// kernel records an error, waits (bounded) for its MMAs, frees TMEM, returns.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "fft_device.cuh"
#include "split_tc.h"

namespace mgb {

namespace {

constexpr int kUThreads = 256;
constexpr int kTmemCols = 64;  // two 128 x 32 FP32 accumulators

// shared-memory layout (bytes)
constexpr int kATile = 128 * 64;                   // 128 rows x 32 bf16 per tile and limb
constexpr int kAOff = 0;                           // [limb][tile] A operands: 3 x 2 x 8 KB
constexpr int kBOff = kAOff + 3 * 2 * kATile;      // [limb] B operands: 3 x 2 KB
constexpr int kXOff = kBOff + 3 * 2048;            // exchange: 4096 points padded
constexpr int kXElems = 4096 + 256;                // upad(4095) + 1
constexpr int kTwOff = kXOff + kXElems * 8;        // 512 stage twiddle factors
constexpr int kBarOff = kTwOff + 512 * 8;          // 3 mbarriers (24 B) + TMEM address (4 B)
constexpr int kUSmem = kBarOff + 64;

__device__ __forceinline__ int upad(int e) { return e + (e >> 4); }

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: canonical K-major layout, no swizzle.
__device__ __forceinline__ unsigned long long umma_desc(unsigned saddr)
{
    unsigned long long d = 0;
    d |= (unsigned long long)((saddr >> 4) & 0x3FFFu);
    d |= (unsigned long long)((128u >> 4) & 0x3FFFu) << 16;  // leading: K-adjacent core matrices
    d |= (unsigned long long)((512u >> 4) & 0x3FFFu) << 32;  // stride: 8-row groups
    d |= 1ull << 46;                                          // descriptor version
    return d;                                                 // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D F32, A and B BF16, both K-major, N = 32, M = 128.
constexpr unsigned kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void umma(unsigned dtmem, unsigned long long ad, unsigned long long bd, unsigned acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(unsigned bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool bar_try_wait(unsigned bar, unsigned parity)
{
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `parity` of the mbarrier.
__device__ __forceinline__ bool bar_wait(unsigned bar, unsigned parity)
{
    for (unsigned i = 0; i < (1u << 22); i++)
        if (bar_try_wait(bar, parity))
            return true;
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&d)[32])
{
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++)
        d[i] = __uint_as_float(r[i]);
}

// (a, b) as LIMBS bf16x2 pairs by truncation: each limb keeps the top 8
// significant bits of what is left, the residual is exact, and three limbs
// hold an FP32 value exactly (24 bits); two keep 16 bits.  The pair of high
// halves is one byte permute.
// Two limbs round to nearest instead (truncation would bias the 16 bits kept).
template <int LIMBS>
__device__ __forceinline__ void split2(float a, float b, unsigned (&o)[LIMBS])
{
    if constexpr (LIMBS == 3) {
        unsigned ua = __float_as_uint(a), ub = __float_as_uint(b);
#pragma unroll
        for (int l = 0; l < LIMBS; l++) {
            o[l] = __byte_perm(ua, ub, 0x7632);  // high half of a (low), high half of b (high)
            if (l + 1 < LIMBS) {
                ua = __float_as_uint(__uint_as_float(ua) - __uint_as_float(ua & 0xFFFF0000u));
                ub = __float_as_uint(__uint_as_float(ub) - __uint_as_float(ub & 0xFFFF0000u));
            }
        }
    } else {
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
}

// Bulk copy of `bytes` contiguous bytes into shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_copy(unsigned dst, const void *src, unsigned bytes, unsigned bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Issues the copies of block `blk`'s transforms into the staging area (thread 0).
template <int N, int T>
__device__ __forceinline__ void prefetch_block(const SplitArgs &a, long long blk, unsigned stage, unsigned bar)
{
    const long long tr0 = blk * T;
    const unsigned nt = (unsigned)((a.ntrans - tr0) < T ? (a.ntrans - tr0) : T);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(nt * (unsigned)(N * sizeof(float2)))
                 : "memory");
    for (unsigned t = 0; t < nt; t++)
        bulk_copy(stage + t * (unsigned)(N * sizeof(float2)), a.in + (tr0 + t) * a.in_dist,
                  (unsigned)(N * sizeof(float2)), bar);
}

template <int S, int LIMBS>
__global__ void __launch_bounds__(kUThreads, 2) split_umma_fft(const SplitArgs a)
{
    constexpr int N = S == 2 ? 256 : 4096;
    constexpr int T = 4096 / N;  // transforms per block of 4096 points
    constexpr int Q = N / 16;    // columns per transform
    constexpr int NT = LIMBS == 3 ? 6 : 3;
    constexpr int ta[6] = {LIMBS == 3 ? 2 : 1, LIMBS == 3 ? 1 : 0, 0, 1, 0, 0};  // F limb
    constexpr int tb[6] = {0, 1, LIMBS == 3 ? 2 : 0, 0, 1, 0};                    // X limb

    extern __shared__ __align__(1024) unsigned char sm[];
    float2 *X = (float2 *)(sm + kXOff);
    float2 *t1 = (float2 *)(sm + kTwOff), *t2 = t1 + 256;
    // mbarriers: [0], [1] MMA completion of tiles 0 and 1, [2] input prefetch
    const unsigned bar0 = smem_u32(sm + kBarOff), bar_in = bar0 + 16;
    unsigned *tmem_slot = (unsigned *)(sm + kBarOff + 24);
    // the next block's input lands in the A-operand region once the last
    // stage's products are done with it
    const float2 *stage_in = (const float2 *)(sm + kAOff);
    const int tid = threadIdx.x, warp = tid >> 5, half = tid >> 7;
    const bool bulk = a.bulk != 0;

    // B operands (F limbs, already in core-matrix order) and stage twiddles
    for (int i = tid; i < 3 * 2048 / 16; i += kUThreads)
        ((uint4 *)(sm + kBOff))[i] = __ldg(&((const uint4 *)a.bfrag)[i]);
    for (int i = tid; i < 512; i += kUThreads)
        t1[i] = __ldg(&a.tw[i]);
    if (tid == 0) {
        for (int b = 0; b < 3; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar0 + 8 * b), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = *tmem_slot;
    unsigned phase = 0, in_phase = 0;
    bool ok = true, in_flight = false;

    const long long nblocks = ((long long)a.ntrans + T - 1) / T;
    if (bulk && tid == 0 && (long long)blockIdx.x < nblocks) {
        prefetch_block<N, T>(a, blockIdx.x, smem_u32(stage_in), bar_in);
        in_flight = true;
    }
    in_flight = __syncthreads_or(in_flight) != 0;
    for (long long blk = blockIdx.x; blk < nblocks && ok; blk += gridDim.x) {
        const long long tr0 = blk * T;
        if (bulk) {
            ok = __syncthreads_and(tid == 0 ? bar_wait(bar_in, in_phase & 1) : true) != 0;
            if (!ok) {
                if (tid == 0 && a.err)
                    atomicExch(a.err, 1);
                break;
            }
            in_phase++;
            in_flight = false;
            for (int e = tid; e < 4096; e += kUThreads) {
                const int t = e / N;
                float2 v = tr0 + t < a.ntrans ? stage_in[e] : make_float2(0.f, 0.f);
                if (a.conj)
                    v.y = -v.y;
                X[upad(e)] = v;
            }
        } else {
            for (int e = tid; e < 4096; e += kUThreads) {
                const int t = e / N, n = e % N;
                float2 v = make_float2(0.f, 0.f);
                if (tr0 + t < a.ntrans)
                    v = __ldg(&a.in[(tr0 + t) * a.in_dist + n]);
                if (a.conj)
                    v.y = -v.y;
                X[upad(e)] = v;
            }
        }
        __syncthreads();

#pragma unroll 1
        for (int s = 0; s < S && ok; s++) {
            const int p = 1 << (4 * s);
            // this thread's column: jj = tid (rows of the two M = 128 tiles)
            const int jj = tid, tt = jj / Q, j = jj % Q;
            float2 x[16];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                float2 v = X[upad(tt * N + j + Q * m)];
                if (s == 1)
                    v = cmul(v, t1[m * 16 + (j & 15)]);
                else if (s == 2)
                    v = cmul(v, cmul(t1[m * 16 + (j >> 4)], t2[m * 16 + (j & 15)]));
                x[m] = v;
            }
            // A rows: chunk c (16 B) of row r holds K = 8c .. 8c+7:
            // c = 0: Xr 0-7, 1: Xr 8-15, 2: Xi 0-7, 3: Xi 8-15
            const int tile = jj >> 7, r = jj & 127;
            unsigned char *arow = sm + kAOff + tile * kATile + (r >> 3) * 512 + (r & 7) * 16;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                unsigned w[4][LIMBS];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int m = (c & 1) * 8 + 2 * q;
                    if (c < 2)
                        split2<LIMBS>(x[m].x, x[m + 1].x, w[q]);
                    else
                        split2<LIMBS>(x[m].y, x[m + 1].y, w[q]);
                }
#pragma unroll
                for (int l = 0; l < LIMBS; l++)
                    *(uint4 *)(arow + l * 2 * kATile + c * 128) = make_uint4(w[0][l], w[1][l], w[2][l], w[3][l]);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            fence_before();
            // each half of the CTA owns one M = 128 tile: its products start as
            // soon as that half has written its operands
            asm volatile("bar.sync %0, 128;" ::"r"(1 + half) : "memory");
            if ((tid & 127) == 0) {
                fence_after();
#pragma unroll
                for (int q = 0; q < NT; q++)
#pragma unroll
                    for (int kh = 0; kh < 2; kh++) {
                        const unsigned aaddr = smem_u32(sm + kAOff + tb[q] * 2 * kATile + half * kATile + kh * 256);
                        const unsigned baddr = smem_u32(sm + kBOff + ta[q] * 2048 + kh * 256);
                        umma(tmem + half * 32, umma_desc(aaddr), umma_desc(baddr), (q | kh) ? 1u : 0u);
                    }
                umma_commit(bar0 + 8 * half);
            }
            // every gather of this stage is done before any scatter below; one
            // thread per half waits for its tile's commit
            ok = __syncthreads_and((tid & 127) == 0 ? bar_wait(bar0 + 8 * half, phase & 1) : true) != 0;
            if (!ok) {
                if (tid == 0 && a.err)
                    atomicExch(a.err, 1);
            } else {
                phase++;
            }
            fence_after();
            if (ok) {
                if (s == S - 1 && bulk && tid == 0 && blk + gridDim.x < nblocks) {
                    // every product of this block is done: the A region is free
                    prefetch_block<N, T>(a, blk + gridDim.x, smem_u32(stage_in), bar_in);
                    in_flight = true;
                }
                // D row of this thread's column: lane group (warp & 3), tile (warp >> 2)
                float d[32];
                tmem_ld32(tmem + ((unsigned)((warp & 3) * 32) << 16) + (warp >> 2) * 32, d);
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int pos = tt * N + (j / p) * 16 * p + (j & (p - 1)) + k * p;
                    X[upad(pos)] = make_float2(d[k], d[16 + k]);
                }
            }
            fence_before();
            __syncthreads();
        }
        if (ok) {
            for (int e = tid; e < 4096; e += kUThreads) {
                const int t = e / N, n = e % N;
                if (tr0 + t < a.ntrans) {
                    float2 v = X[upad(e)];
                    if (a.conj)
                        v.y = -v.y;
                    a.out[(tr0 + t) * a.out_dist + n] = v;
                }
            }
        }
        in_flight = __syncthreads_or(in_flight) != 0;
    }
    if (!ok) {
        // let this CTA's products and copies drain before TMEM is released
        // (bounded): the timed-out phases are still `phase` / `in_phase`
        if (tid == 0) {
            bar_wait(bar0, phase & 1);
            bar_wait(bar0 + 8, phase & 1);
            if (in_flight)
                bar_wait(bar_in, in_phase & 1);
        }
        __syncthreads();
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
    }
}

double bf16r(double v)
{
    float f = (float)v;
    unsigned u;
    std::memcpy(&u, &f, 4);
    u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return (double)f;
}

}  // namespace

const void *split_umma_kernel(int stages, int limbs)
{
    if (stages == 2)
        return limbs == 3 ? (const void *)&split_umma_fft<2, 3> : (const void *)&split_umma_fft<2, 2>;
    if (stages == 3)
        return limbs == 3 ? (const void *)&split_umma_fft<3, 3> : (const void *)&split_umma_fft<3, 2>;
    return nullptr;
}

size_t split_umma_smem_bytes() { return (size_t)kUSmem; }
int split_umma_threads() { return kUThreads; }

std::vector<unsigned short> split_umma_bfrag_table()
{
    // [limb][core matrix (g = n/8, c = kk/8) at (4g + c) * 128 B][row n % 8][kk % 8], bf16 bits
    std::vector<unsigned short> t(3 * 1024);
    for (int n = 0; n < 32; n++)
        for (int kk = 0; kk < 32; kk++) {
            const int k = n & 15, m = kk & 15;
            const double ph = -2.0 * M_PI * (double)((k * m) % 16) / 16.0;
            const double re = std::cos(ph), im = std::sin(ph);
            double v = (n < 16) ? (kk < 16 ? re : -im) : (kk < 16 ? im : re);
            for (int l = 0; l < 3; l++) {
                const double h = bf16r(v);
                v -= h;
                float f = (float)h;
                unsigned u;
                std::memcpy(&u, &f, 4);
                const int idx = l * 1024 + ((n >> 3) * 4 + (kk >> 3)) * 64 + (n & 7) * 8 + (kk & 7);
                t[idx] = (unsigned short)(u >> 16);
            }
        }
    return t;
}

}  // namespace mgb
