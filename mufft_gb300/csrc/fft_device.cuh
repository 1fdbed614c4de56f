// Device building blocks of the GB300 FFT: complex arithmetic, register DFTs
// of size 2/4/8/16 and the tile-FFT kernel template used by every pass.
//
// Algorithm (the GPU form of muFFT's Stockham autosort passes,
// kernel.c:151-453): a transform of length L is a sequence of radix-r
// Stockham stages.  In stage s with sub-transform size p, butterfly i takes the
// r inputs at i + m*L/r, multiplies input m by W_{rp}^(m*k) with k = i mod p,
// runs a DFT of size r and stores output m' at (i - k)*r + k + m'*p.  After
// the last stage the result is in natural order, so no bit reversal is needed.
//
// GB300 mapping: one CTA runs C transforms.  Every thread owns R elements
// (R/r butterflies per stage) in registers; stage 0 loads straight from HBM,
// the last stage stores straight to HBM, and the stages in between exchange
// through padded shared memory.  Each transform therefore makes exactly one
// read and one write pass over HBM.
#pragma once

#include "common.h"

namespace mgb {

// ------------------------------------------------------------ complex math

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 mul_neg_i(float2 a) { return make_float2(a.y, -a.x); }

// Constants of the 8th and 16th roots of unity.
constexpr float kRsqrt2 = 0.70710678118654752440f;
constexpr float kCos8 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float kSin8 = 0.38268343236508977173f;  // sin(pi/8)

// x * exp(-i*pi/4), x * exp(-3i*pi/4)
__device__ __forceinline__ float2 mul_w8_1(float2 a) { return make_float2(kRsqrt2 * (a.x + a.y), kRsqrt2 * (a.y - a.x)); }
__device__ __forceinline__ float2 mul_w8_3(float2 a) { return make_float2(kRsqrt2 * (a.y - a.x), -kRsqrt2 * (a.x + a.y)); }

// ------------------------------------------------------- register DFTs
// Forward DFTs (W = exp(-2*pi*i/r)), natural order in and out.

__device__ __forceinline__ void dft2(float2 &a, float2 &b)
{
    float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

__device__ __forceinline__ void dft4(float2 &x0, float2 &x1, float2 &x2, float2 &x3)
{
    float2 t0 = cadd(x0, x2), t1 = csub(x0, x2);
    float2 t2 = cadd(x1, x3), t3 = mul_neg_i(csub(x1, x3));
    x0 = cadd(t0, t2);
    x2 = csub(t0, t2);
    x1 = cadd(t1, t3);
    x3 = csub(t1, t3);
}

template <int r> struct Dft;

template <> struct Dft<1> {
    __device__ __forceinline__ static void run(float2 *) {}
};

template <> struct Dft<2> {
    __device__ __forceinline__ static void run(float2 *v) { dft2(v[0], v[1]); }
};

template <> struct Dft<4> {
    __device__ __forceinline__ static void run(float2 *v) { dft4(v[0], v[1], v[2], v[3]); }
};

template <> struct Dft<8> {
    __device__ __forceinline__ static void run(float2 *v)
    {
        dft4(v[0], v[2], v[4], v[6]);  // even samples -> E_k at v[2k]
        dft4(v[1], v[3], v[5], v[7]);  // odd samples  -> O_k at v[2k+1]
        float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
        float2 o0 = v[1], o1 = mul_w8_1(v[3]), o2 = mul_neg_i(v[5]), o3 = mul_w8_3(v[7]);
        v[0] = cadd(e0, o0);
        v[4] = csub(e0, o0);
        v[1] = cadd(e1, o1);
        v[5] = csub(e1, o1);
        v[2] = cadd(e2, o2);
        v[6] = csub(e2, o2);
        v[3] = cadd(e3, o3);
        v[7] = csub(e3, o3);
    }
};

template <> struct Dft<16> {
    __device__ __forceinline__ static void run(float2 *v)
    {
        // 4 x 4: DFT-4 over n = b + 4a for each b, twiddle W16^(b*q), DFT-4 over b.
        dft4(v[0], v[4], v[8], v[12]);
        dft4(v[1], v[5], v[9], v[13]);
        dft4(v[2], v[6], v[10], v[14]);
        dft4(v[3], v[7], v[11], v[15]);
        const float2 w1 = make_float2(kCos8, -kSin8);
        const float2 w3 = make_float2(kSin8, -kCos8);
        const float2 w9 = make_float2(-kCos8, kSin8);
        v[5] = cmul(v[5], w1);
        v[9] = mul_w8_1(v[9]);
        v[13] = cmul(v[13], w3);
        v[6] = mul_w8_1(v[6]);
        v[10] = mul_neg_i(v[10]);
        v[14] = mul_w8_3(v[14]);
        v[7] = cmul(v[7], w3);
        v[11] = mul_w8_3(v[11]);
        v[15] = cmul(v[15], w9);
        dft4(v[0], v[1], v[2], v[3]);
        dft4(v[4], v[5], v[6], v[7]);
        dft4(v[8], v[9], v[10], v[11]);
        dft4(v[12], v[13], v[14], v[15]);
        // y[q + 4s] now sits at v[4q + s]: transpose the 4x4 block.
        float2 t;
        t = v[1]; v[1] = v[4]; v[4] = t;
        t = v[2]; v[2] = v[8]; v[8] = t;
        t = v[3]; v[3] = v[12]; v[12] = t;
        t = v[6]; v[6] = v[9]; v[9] = t;
        t = v[7]; v[7] = v[13]; v[13] = t;
        t = v[11]; v[11] = v[14]; v[14] = t;
    }
};

// ------------------------------------------------------------- schedule

constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }

// Stage plan of a length-L transform whose threads own R elements each:
// radix-16 stages, then one smaller stage for the leftover factor.
template <int L, int R> struct Sched {
    static_assert(L >= 2 && (L & (L - 1)) == 0, "power of two");
    static_assert(R <= L && L % R == 0, "R divides L");
    static constexpr int T = L / R;                  // threads per transform
    static constexpr int LOG = ilog2c(L);
    static constexpr int NFULL = L < 16 ? 0 : LOG / 4;
    static constexpr int REMB = L < 16 ? LOG : LOG % 4;
    static constexpr int NST = NFULL + (REMB ? 1 : 0);
    __host__ __device__ static constexpr int radix(int s) { return s < NFULL ? 16 : (1 << REMB); }
    __host__ __device__ static constexpr int pbefore(int s)
    {
        int p = 1;
        for (int i = 0; i < s; i++)
            p *= radix(i);
        return p;
    }
};

// Shared-memory words per transform.  Positions are padded by one slot every
// 16 (pos + pos/16) so that radix-16 strided writes spread over all banks; an
// extra offset makes the region stride ≡ 16/C (mod 16) so that the 16 lanes of
// a half-warp walking ACROSS C transforms hit 16 distinct bank pairs.
template <int L, int C, bool ACROSS_USED>
__host__ __device__ constexpr int region_stride()
{
    if (L < 16)
        return L;
    int base = L + L / 16;
    if (!ACROSS_USED || C < 2)
        return base;
    int want = C >= 16 ? 1 : 16 / C;  // 64-bit accesses are served per half-warp
    int have = base % 16;
    return base + ((want - have + 16) % 16);
}

__device__ __forceinline__ int padpos(int pos) { return pos + (pos >> 4); }

template <int MAP, int C, int T>
__device__ __forceinline__ void split_tid(int tid, int &c, int &t)
{
    if (MAP == ALONG) {
        t = tid % T;
        c = tid / T;
    } else {
        c = tid % C;
        t = tid / C;
    }
}

// ---------------------------------------------------------------- stages

// Twiddle multiply and DFT of stage s on the thread's R registers.
// Register j*r + m holds input m of butterfly i = t + j*T.
template <int L, int R, int s>
__device__ __forceinline__ void stage_compute(float2 (&v)[R], int t, const float2 *__restrict__ tw)
{
    using S = Sched<L, R>;
    constexpr int r = S::radix(s), p = S::pbefore(s), NB = R / r, T = S::T;
#pragma unroll
    for (int j = 0; j < NB; j++) {
        if constexpr (p > 1) {
            const int i = t + j * T;
            const int k = i & (p - 1);
            const float4 *e = reinterpret_cast<const float4 *>(tw + stage_table_base(r, p) + 4 * k);
            const float4 a = __ldg(e);
            float2 w[16];
            w[1] = make_float2(a.x, a.y);
            w[2] = make_float2(a.z, a.w);
            if constexpr (r > 4) {
                const float4 b = __ldg(e + 1);
                w[4] = make_float2(b.x, b.y);
                w[8] = make_float2(b.z, b.w);
            }
            // remaining powers: at most three rounded products deep
#pragma unroll
            for (int m = 3; m < r; m++) {
                if (m == 4 || m == 8)
                    continue;
                const int hi = m >= 8 ? 8 : (m >= 4 ? 4 : 2);
                w[m] = cmul(w[m - hi], w[hi]);
            }
#pragma unroll
            for (int m = 1; m < r; m++)
                v[j * r + m] = cmul(v[j * r + m], w[m]);
        }
        Dft<r>::run(&v[j * r]);
    }
}

// Store the outputs of stage s to the transform's shared-memory region.
// Output m of butterfly i goes to (i - k)*r + k + m*p.  When p is a multiple
// of 16 the padded address of that position is padpos(base) + m*(p + p/16),
// and for p == 1, r == 16 it is 17*i + m, so the inner loop is a base plus
// compile-time offsets.
template <int L, int R, int s>
__device__ __forceinline__ void stage_write(float2 *region, const float2 (&v)[R], int t)
{
    using S = Sched<L, R>;
    constexpr int r = S::radix(s), p = S::pbefore(s), NB = R / r, T = S::T;
#pragma unroll
    for (int j = 0; j < NB; j++) {
        const int i = t + j * T;
        if constexpr (p % 16 == 0) {
            const int k = i & (p - 1);
            float2 *b = region + padpos((i - k) * r + k);
#pragma unroll
            for (int m = 0; m < r; m++)
                b[m * (p + p / 16)] = v[j * r + m];
        } else if constexpr (p == 1 && r == 16) {
            float2 *b = region + 17 * i;
#pragma unroll
            for (int m = 0; m < r; m++)
                b[m] = v[j * r + m];
        } else {
            const int k = i & (p - 1);
            const int base = (i - k) * r + k;
#pragma unroll
            for (int m = 0; m < r; m++)
                region[padpos(base + m * p)] = v[j * r + m];
        }
    }
}

// Load the inputs of stage s from the transform's shared-memory region:
// register j*r + m <- position t + T*(j + m*NB).
template <int L, int R, int s>
__device__ __forceinline__ void stage_read(const float2 *region, float2 (&v)[R], int t)
{
    using S = Sched<L, R>;
    constexpr int r = S::radix(s), NB = R / r, T = S::T;
    if constexpr (T % 16 == 0) {
        const float2 *b = region + padpos(t);
#pragma unroll
        for (int j = 0; j < NB; j++)
#pragma unroll
            for (int m = 0; m < r; m++)
                v[j * r + m] = b[(j + m * NB) * (T + T / 16)];
    } else {
#pragma unroll
        for (int j = 0; j < NB; j++)
#pragma unroll
            for (int m = 0; m < r; m++)
                v[j * r + m] = region[padpos(t + T * (j + m * NB))];
    }
}

// ------------------------------------------------------ prologue / epilogue

__device__ __forceinline__ float2 c2r_fixup(float2 a, float2 bm, float2 w)
{
    float2 b = cconj(bm);
    return cadd(cadd(a, b), cmul(csub(a, b), w));
}

// Stage-0 load: register j*r + m <- element t + T*(j + m*NB) of transform
// `tr` (slot q = j + m*NB).  ALONG loads have unit stride (the planner only
// builds them that way), so addresses are a base plus constant offsets.
template <int L, int R, int LMAP>
__device__ __forceinline__ void load_stage0(const TileArgs &a, const float2 *__restrict__ in,
                                            const float2 *__restrict__ in2, unsigned tr, int t,
                                            float2 (&v)[R])
{
    using S = Sched<L, R>;
    constexpr int r = S::radix(0), NB = R / r, T = S::T;
#pragma unroll
    for (int q = 0; q < R; q++)
        v[q] = make_float2(0.f, 0.f);
    if (tr >= a.ntrans)
        return;
    const int nq = a.half ? R / 2 : R;  // zero-padded upper half: slots q >= R/2 stay zero
    const long long tbase = (long long)tr * a.in_dist;
    const long long step = (LMAP == ALONG) ? (long long)T : (long long)T * a.in_stride;
    const long long first = tbase + ((LMAP == ALONG) ? (long long)t : (long long)t * a.in_stride);
    switch (a.prologue) {
    case PRO_PLAIN: {
        const float2 *p0 = in + first;
#pragma unroll
        for (int j = 0; j < NB; j++)
#pragma unroll
            for (int m = 0; m < r; m++) {
                const int q = j + m * NB;
                if (q < nq)
                    v[j * r + m] = __ldg(p0 + q * step);
            }
        break;
    }
    case PRO_MUL: {
        const float2 *p0 = in + first, *p1 = in2 + first;
#pragma unroll
        for (int j = 0; j < NB; j++)
#pragma unroll
            for (int m = 0; m < r; m++) {
                const int q = j + m * NB;
                if (q < nq)
                    v[j * r + m] = cscale(cmul(__ldg(p0 + q * step), __ldg(p1 + q * step)), a.scale);
            }
        break;
    }
    default: {
        // c2r fix-ups: X[local] and X[M - local] with local = tr*ldist + pos*stride
        const long long tb = tbase - (long long)tr * a.mirror_ldist;
        const long long lfirst = (long long)tr * a.mirror_ldist + (long long)t * a.in_stride;
        const long long lstep = (long long)T * a.in_stride;
        const bool mul = a.prologue == PRO_MUL_C2R;
#pragma unroll
        for (int j = 0; j < NB; j++)
#pragma unroll
            for (int m = 0; m < r; m++) {
                const int q = j + m * NB;
                if (q < nq) {
                    const long long local = lfirst + q * lstep;
                    const long long ia = tb + local, ib = tb + a.mirror_len - local;
                    float2 xa = __ldg(&in[ia]), xb = __ldg(&in[ib]);
                    if (mul) {
                        xa = cscale(cmul(xa, __ldg(&in2[ia])), a.scale);
                        xb = cscale(cmul(xb, __ldg(&in2[ib])), a.scale);
                    }
                    v[j * r + m] = c2r_fixup(xa, xb, __ldg(&a.rtw[local]));
                }
            }
        break;
    }
    }
    if (a.conj & 1) {
#pragma unroll
        for (int q = 0; q < R; q++)
            v[q].y = -v[q].y;
    }
}

// W_N^m = exp(-2*pi*i*m/N) for m < N <= 2^28, scale = 2/N.  sincospif gets
// an exactly representable argument: m itself when m < 2^24, otherwise the
// product of the twiddles of m's high and low 12-bit parts.
__device__ __forceinline__ float2 fourstep_twiddle(unsigned m, float scale)
{
    float s, c;
    if (m < (1u << 24)) {
        sincospif((float)m * scale, &s, &c);
        return make_float2(c, -s);
    }
    float s2, c2;
    sincospif((float)(m & ~4095u) * scale, &s, &c);
    sincospif((float)(m & 4095u) * scale, &s2, &c2);
    return cmul(make_float2(c, -s), make_float2(c2, -s2));
}

// Real-to-complex fix-up of bin k from Z[k] and Z[M-k] (kernel.c:47-82).
__device__ __forceinline__ void r2c_bins(float2 zk, float2 zmk, float2 w, float2 &lo, float2 &hi)
{
    float2 b = cconj(zmk);
    float2 fe = cadd(zk, b);
    float2 fo = cmul(w, csub(zk, b));
    lo = cscale(cadd(fe, fo), 0.5f);
    hi = cscale(csub(fe, fo), 0.5f);
}

// --------------------------------------------------------------- kernel

template <int L, int R, int C, int LMAP, int SMAP, int s>
__device__ __forceinline__ void run_stages(float2 (&v)[R], int &c, int &t, float2 *smem,
                                           const float2 *__restrict__ tw)
{
    using S = Sched<L, R>;
    if constexpr (s < S::NST) {
        constexpr int RS = region_stride<L, C, (LMAP == ACROSS || SMAP == ACROSS)>();
        stage_write<L, R, s - 1>(smem + c * RS, v, t);
        __syncthreads();
        split_tid<(s == S::NST - 1) ? SMAP : ALONG, C, S::T>(threadIdx.x, c, t);
        stage_read<L, R, s>(smem + c * RS, v, t);
        if (s < S::NST - 1)
            __syncthreads();
        stage_compute<L, R, s>(v, t, tw);
        run_stages<L, R, C, LMAP, SMAP, s + 1>(v, c, t, smem, tw);
    }
}

template <int L, int R, int C, int LMAP, int SMAP>
__global__ void __launch_bounds__(C *(L / R)) tile_fft(const TileArgs a)
{
    using S = Sched<L, R>;
    constexpr int T = S::T, NST = S::NST;
    constexpr int RS = region_stride<L, C, (LMAP == ACROSS || SMAP == ACROSS)>();
    static_assert(NST > 1 || LMAP == SMAP, "single-stage tiles cannot change the thread map");
    extern __shared__ float2 smem[];

    const float2 *in = a.in + (long long)blockIdx.y * a.in_batch;
    const float2 *in2 = a.in2 ? a.in2 + (long long)blockIdx.y * a.in_batch : nullptr;
    float2 *out = a.out + (long long)blockIdx.y * a.out_batch;
    const unsigned tile0 = blockIdx.x * C;

    float2 v[R];
    int c, t;
    split_tid<LMAP, C, T>(threadIdx.x, c, t);
    load_stage0<L, R, LMAP>(a, in, in2, tile0 + c, t, v);
    stage_compute<L, R, 0>(v, t, a.tw);
    run_stages<L, R, C, LMAP, SMAP, 1>(v, c, t, smem, a.tw);

    // Last stage: register j*r + m holds output t + T*(j + m*NB).
    constexpr int rl = S::radix(NST - 1), NBL = R / rl;
    const unsigned tr = tile0 + c;
    const bool valid = tr < a.ntrans;
    const long long obase = (long long)tr * a.out_dist;

    if (a.epilogue == EPI_R2C || a.epilogue == EPI_R2C_FULL) {
        // Z[k] and Z[L-k] sit in different threads: go through shared memory.
        constexpr int M = L;
        const bool full = a.epilogue == EPI_R2C_FULL;
        if constexpr (NST > 1) {
            float2 *region = smem + c * RS;
            __syncthreads();
#pragma unroll
            for (int j = 0; j < NBL; j++)
#pragma unroll
                for (int m = 0; m < rl; m++)
                    region[padpos(t + T * (j + m * NBL))] = v[j * rl + m];
            __syncthreads();
            if (valid) {
#pragma unroll
                for (int q = 0; q < R; q++) {
                    const int k = t + T * q;
                    float2 zk = region[padpos(k)];
                    if (k == 0) {
                        out[obase] = make_float2(zk.x + zk.y, 0.f);
                        out[obase + (long long)M * a.out_stride] = make_float2(zk.x - zk.y, 0.f);
                    } else {
                        float2 lo, hi;
                        r2c_bins(zk, region[padpos(M - k)], __ldg(&a.rtw[k]), lo, hi);
                        out[obase + (long long)k * a.out_stride] = lo;
                        if (full)
                            out[obase + (long long)(k + M) * a.out_stride] = hi;
                    }
                }
            }
        } else {
            // One thread owns the whole transform (L <= 16): natural order in v.
            if (valid) {
                out[obase] = make_float2(v[0].x + v[0].y, 0.f);
                out[obase + (long long)M * a.out_stride] = make_float2(v[0].x - v[0].y, 0.f);
#pragma unroll
                for (int k = 1; k < M; k++) {
                    float2 lo, hi;
                    r2c_bins(v[k], v[M - k], __ldg(&a.rtw[k]), lo, hi);
                    out[obase + (long long)k * a.out_stride] = lo;
                    if (full)
                        out[obase + (long long)(k + M) * a.out_stride] = hi;
                }
            }
        }
        return;
    }

    if (!valid)
        return;
    const long long ostep = (SMAP == ALONG) ? (long long)T : (long long)T * a.out_stride;
    float2 *o0 = out + obase + ((SMAP == ALONG) ? (long long)t : (long long)t * a.out_stride);
    if (a.epilogue == EPI_TWIDDLE) {
#pragma unroll
        for (int j = 0; j < NBL; j++)
#pragma unroll
            for (int m = 0; m < rl; m++) {
                const int q = j + m * NBL;
                float2 y = cmul(v[j * rl + m], fourstep_twiddle((unsigned)(t + T * q) * tr, a.tw_scale));
                if (a.conj & 2)
                    y.y = -y.y;
                o0[q * ostep] = y;
            }
    } else {
        const float sg = (a.conj & 2) ? -1.f : 1.f;
#pragma unroll
        for (int j = 0; j < NBL; j++)
#pragma unroll
            for (int m = 0; m < rl; m++) {
                const int q = j + m * NBL;
                const float2 y = v[j * rl + m];
                o0[q * ostep] = make_float2(y.x, sg * y.y);
            }
    }
}

// Shared memory bytes a tile_fft instantiation needs.
template <int L, int R, int C, int LMAP, int SMAP>
constexpr size_t tile_smem_bytes()
{
    return (Sched<L, R>::NST > 1)
               ? (size_t)C * region_stride<L, C, (LMAP == ACROSS || SMAP == ACROSS)>() * sizeof(float2)
               : 0;
}

}  // namespace mgb
