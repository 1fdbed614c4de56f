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

#include <cooperative_groups.h>

#include "common.h"

namespace mgb {

namespace cg = cooperative_groups;

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

// A tile is C transforms of length L spread over a cluster of Q CTAs: CTA
// rank j owns positions [j*L/Q, (j+1)*L/Q) of every transform in its shared
// memory and, in stage s (radix r), butterflies [j*B, (j+1)*B) with
// B = L/(r*Q).  Thread tl of a transform runs butterflies j*B + tl + TL*u,
// u < R/r.  When B is a multiple of the stage's sub-transform size p, the
// outputs (i - k)*r + k + m*p of those butterflies fall in the CTA's own
// slice, so every stage writes locally and reads its inputs i + m*L/r from
// whichever CTA owns them (distributed shared memory when Q > 1).
template <int L, int R, int Q> struct Tile {
    using S = Sched<L, R>;
    static constexpr int TL = L / (R * Q);  // threads per transform per CTA
    static constexpr int LQ = L / Q;        // positions per CTA per transform
    static_assert(TL >= 1 && L % (R * Q) == 0, "R*Q must divide L");
    __host__ __device__ static constexpr int B(int s) { return L / (S::radix(s) * Q); }
    __host__ __device__ static constexpr bool local_writes()
    {
        for (int s = 0; s + 1 < S::NST; s++)
            if (B(s) % S::pbefore(s) != 0)
                return false;
        return true;
    }
    static_assert(Q == 1 || local_writes(), "stage outputs must stay in the writing CTA");
};

// Shared-memory words per transform slice.  Positions are padded by one slot
// every 16 (pos + pos/16) so that radix-16 strided writes spread over all
// banks; an extra offset makes the slice stride ≡ 16/C (mod 16) so that the
// 16 lanes of a half-warp walking ACROSS C transforms hit 16 distinct bank
// pairs (64-bit accesses are served per half-warp).
template <int LQ, int C, bool ACROSS_USED>
__host__ __device__ constexpr int region_stride()
{
    if (LQ < 16)
        return LQ;
    int base = LQ + LQ / 16;
    if (!ACROSS_USED || C < 2)
        return base;
    int want = C >= 16 ? 1 : 16 / C;
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

template <int Q>
__device__ __forceinline__ void tile_sync()
{
    if constexpr (Q > 1)
        cg::this_cluster().sync();
    else
        __syncthreads();
}

// ---------------------------------------------------------------- stages

// Twiddle multiply and DFT of stage s on the thread's R registers.
// Register u*r + m holds input m of butterfly i = j*B + tl + TL*u.
template <int L, int R, int Q, int s>
__device__ __forceinline__ void stage_compute(float2 (&v)[R], int j, int tl, const float2 *__restrict__ tw)
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, Q>;
    constexpr int r = S::radix(s), p = S::pbefore(s), NB = R / r;
#pragma unroll
    for (int u = 0; u < NB; u++) {
        if constexpr (p > 1) {
            const int i = j * TT::B(s) + tl + TT::TL * u;
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
                v[u * r + m] = cmul(v[u * r + m], w[m]);
        }
        Dft<r>::run(&v[u * r]);
    }
}

// Store the outputs of stage s into the CTA's own slice (local offset
// pos - j*LQ).  Output m of butterfly i goes to (i - k)*r + k + m*p; when p
// is a multiple of 16 the padded address is padpos(base) + m*(p + p/16), and
// for p == 1, r == 16 it is 17*(i - j*LQ/16) + m: a base plus constants.
template <int L, int R, int Q, int s>
__device__ __forceinline__ void stage_write(float2 *region, const float2 (&v)[R], int j, int tl)
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, Q>;
    constexpr int r = S::radix(s), p = S::pbefore(s), NB = R / r;
#pragma unroll
    for (int u = 0; u < NB; u++) {
        const int i = j * TT::B(s) + tl + TT::TL * u;
        if constexpr (p % 16 == 0) {
            const int k = i & (p - 1);
            float2 *b = region + padpos((i - k) * r + k - j * TT::LQ);
#pragma unroll
            for (int m = 0; m < r; m++)
                b[m * (p + p / 16)] = v[u * r + m];
        } else if constexpr (p == 1 && r == 16) {
            float2 *b = region + 17 * (i - j * (TT::LQ / 16));
#pragma unroll
            for (int m = 0; m < r; m++)
                b[m] = v[u * r + m];
        } else {
            const int k = i & (p - 1);
            const int base = (i - k) * r + k - j * TT::LQ;
#pragma unroll
            for (int m = 0; m < r; m++)
                region[padpos(base + m * p)] = v[u * r + m];
        }
    }
}

// Load the inputs of stage s: register u*r + m <- position i + m*L/r, which
// is local offset B*((j + m*Q) % r) + tl + TL*u in the slice of CTA
// (j + m*Q) / r.
template <int L, int R, int Q, int s>
__device__ __forceinline__ void stage_read(float2 *region, float2 (&v)[R], int j, int tl)
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, Q>;
    constexpr int r = S::radix(s), NB = R / r, B = TT::B(s), TL = TT::TL;
    if constexpr (Q == 1 && TL % 16 == 0 && B % 16 == 0) {
        const float2 *b = region + padpos(tl);
#pragma unroll
        for (int u = 0; u < NB; u++)
#pragma unroll
            for (int m = 0; m < r; m++)
                v[u * r + m] = b[(B * m + TL * u) / 16 * 17];
    } else if constexpr (TL % 16 == 0 && B % 16 == 0 && r % Q == 0) {
        // Q divides r and j < Q: input m lives in CTA (m*Q)/r at local offset
        // B*j + B*((m*Q) % r) + tl + TL*u -- compile-time owners and offsets.
        const int lbase = padpos(B * j + tl);
#pragma unroll
        for (int m = 0; m < r; m++) {
            const int owner = (m * Q) / r;
            const int lq = (m * Q) % r;
            const float2 *b = cg::this_cluster().map_shared_rank(region, owner) + lbase + B * lq + B * lq / 16;
#pragma unroll
            for (int u = 0; u < NB; u++)
                v[u * r + m] = b[TL * u + TL * u / 16];
        }
    } else {
#pragma unroll
        for (int m = 0; m < r; m++) {
            const int owner = (j + m * Q) / r;
            const int lq = (j + m * Q) % r;
            const float2 *b = Q > 1 ? cg::this_cluster().map_shared_rank(region, owner) : region;
#pragma unroll
            for (int u = 0; u < NB; u++)
                v[u * r + m] = b[padpos(B * lq + tl + TL * u)];
        }
    }
}

// ------------------------------------------------------ prologue / epilogue

__device__ __forceinline__ float2 c2r_fixup(float2 a, float2 bm, float2 w)
{
    float2 b = cconj(bm);
    return cadd(cadd(a, b), cmul(csub(a, b), w));
}

// Stage-0 load: register u*r + m <- element p = j*B + tl + TL*u + m*Q*B of
// transform `tr`.  ALONG loads have unit stride (the planner only builds them
// that way), so addresses are a base plus constant offsets.
// Global loads: read-only path, or (COH) L2-coherent loads for data written
// earlier in the same launch by other CTAs.
template <bool COH>
__device__ __forceinline__ float2 gload(const float2 *p)
{
    if constexpr (COH)
        return __ldcg(p);
    else
        return __ldg(p);
}

// L2 cache policies (createpolicy) and the loads / stores that carry them.
__device__ __forceinline__ unsigned long long l2_evict_first()
{
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ unsigned long long l2_evict_last()
{
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ unsigned long long l2_evict_normal()
{
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ float2 ld_policy(const float2 *p, unsigned long long pol)
{
    float2 v;
    asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_policy(float2 *p, float2 v, unsigned long long pol)
{
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
                 : "memory");
}

template <int L, int R, int Q, int LMAP, bool COH = false>
__device__ __forceinline__ void load_stage0(const TileArgs &a, const float2 *__restrict__ in,
                                            const float2 *__restrict__ in2, unsigned tr, int j, int tl,
                                            float2 (&v)[R])
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, Q>;
    constexpr int r = S::radix(0), NB = R / r, B = TT::B(0), TL = TT::TL;
#pragma unroll
    for (int q = 0; q < R; q++)
        v[q] = make_float2(0.f, 0.f);
    if (tr >= a.ntrans)
        return;
    const int mlim = a.half ? r / 2 : r;  // zero-padded upper half: inputs m >= r/2 stay zero
    const long long tbase = (long long)tr * a.in_dist;
    const long long p0 = (long long)j * B + tl;  // position of register 0
    const long long sst = (LMAP == ALONG) ? 1 : a.in_stride;
    const float2 *f = in + tbase + p0 * sst;
    switch (a.prologue) {
    case PRO_PLAIN: {
        // read-only loads carry an L2 policy: evict-first for a pass that
        // streams its input, else evict-normal
        unsigned long long pol = 0;
        if constexpr (!COH)
            pol = (a.l2 & L2_LOAD_FIRST) ? l2_evict_first() : l2_evict_normal();
#pragma unroll
        for (int u = 0; u < NB; u++)
#pragma unroll
            for (int m = 0; m < r; m++)
                if (m < mlim) {
                    const float2 *src = f + (long long)(TL * u + m * Q * B) * sst;
                    if constexpr (COH)
                        v[u * r + m] = gload<COH>(src);
                    else
                        v[u * r + m] = ld_policy(src, pol);
                }
        break;
    }
    case PRO_MUL: {
        const float2 *g = in2 + ((a.in2_bcast & 2) ? 0 : tbase) + p0 * sst;
#pragma unroll
        for (int u = 0; u < NB; u++)
#pragma unroll
            for (int m = 0; m < r; m++)
                if (m < mlim) {
                    const long long o = (long long)(TL * u + m * Q * B) * sst;
                    float2 gv = gload<COH>(g + o);
                    gv.y = a.conj2 ? -gv.y : gv.y;
                    v[u * r + m] = cscale(cmul(gload<COH>(f + o), gv), a.scale);
                }
        break;
    }
    default: {
        // c2r fix-ups: X[local] and X[M - local] with local = tr*ldist + pos*stride
        const long long tb = tbase - (long long)tr * a.mirror_ldist;
        const long long lfirst = (long long)tr * a.mirror_ldist + p0 * a.in_stride;
        const bool mul = a.prologue == PRO_MUL_C2R;
#pragma unroll
        for (int u = 0; u < NB; u++)
#pragma unroll
            for (int m = 0; m < r; m++)
                if (m < mlim) {
                    const long long local = lfirst + (long long)(TL * u + m * Q * B) * a.in_stride;
                    const long long ia = tb + local, ib = tb + a.mirror_len - local;
                    float2 xa = gload<COH>(&in[ia]), xb = gload<COH>(&in[ib]);
                    if (mul) {
                        const long long i2 = (a.in2_bcast & 2) ? tb : 0;  // (single-pass: tb is the transform's base)
                        float2 ga = gload<COH>(&in2[ia - i2]), gb = gload<COH>(&in2[ib - i2]);
                        if (a.conj2) {
                            ga.y = -ga.y;
                            gb.y = -gb.y;
                        }
                        xa = cscale(cmul(xa, ga), a.scale);
                        xb = cscale(cmul(xb, gb), a.scale);
                    }
                    v[u * r + m] = c2r_fixup(xa, xb, __ldg(&a.rtw[local]));
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

// c2r fix-up prologue of a row tile (unit stride, mirror within the row):
// element n of transform tr needs X[n] and X[M - n], which another thread
// loads.  Conditions: prologue PRO_C2R or PRO_MUL_C2R, unit stride,
// mirror_ldist 0, mirror_len L, no `half`.  The row is staged once, coalesced, in the transform's exchange
// slice (padded positions), and both operands are read from there -- one
// global load per element instead of two.  X[M] (needed by n = 0 only) is
// loaded into a register of thread 0 beside the staged values.  PRO_MUL_C2R multiplies by s * B[n] while staging.  Not
// for zero-padded inputs (`half`).  The caller's CTA must not use the slice
// until the next barrier.
template <int L, int R, bool COH>
__device__ __forceinline__ void load_stage0_c2r_rows(const TileArgs &a, const float2 *__restrict__ in,
                                                     const float2 *__restrict__ in2, unsigned tr, int tl,
                                                     float2 *region, float2 (&v)[R])
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, 1>;
    constexpr int r = S::radix(0), NB = R / r, B = TT::B(0), TL = TT::TL;
    const bool valid = tr < a.ntrans;
    const bool mul = a.prologue == PRO_MUL_C2R;
    const long long tbase = (long long)tr * a.in_dist;
    auto fetch = [&](long long n) {
        float2 xv = gload<COH>(in + tbase + n);
        if (mul) {
            float2 g = gload<COH>(in2 + ((a.in2_bcast & 2) ? 0 : tbase) + n);
            g.y = a.conj2 ? -g.y : g.y;
            xv = cscale(cmul(xv, g), a.scale);
        }
        return xv;
    };
    // X[M], the mirror of position 0, is loaded with the staged values so
    // that its latency is not paid after the barrier
    float2 xm = make_float2(0.f, 0.f);
    if (valid) {
#pragma unroll
        for (int i = 0; i < R; i++)
            region[padpos(tl + TL * i)] = fetch(tl + TL * i);
        if (tl == 0)
            xm = fetch(L);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < R; q++)
        v[q] = make_float2(0.f, 0.f);
    if (valid) {
#pragma unroll
        for (int u = 0; u < NB; u++)
#pragma unroll
            for (int m = 0; m < r; m++) {
                const int local = tl + TL * u + m * B;
                const float2 xa = region[padpos(local)];
                // only register 0 of thread 0 is position 0 (its mirror X[M] is not staged)
                const float2 xb = (u == 0 && m == 0 && tl == 0) ? xm : region[padpos(L - local)];
                v[u * r + m] = c2r_fixup(xa, xb, __ldg(&a.rtw[local]));
            }
    }
    if (a.conj & 1) {
#pragma unroll
        for (int q = 0; q < R; q++)
            v[q].y = -v[q].y;
    }
}

// Stage-0 inputs of a column tile already staged in shared memory (by TMA):
// element n of the tile's column c at sin[n*C + c].  Plain prologue only.
template <int L, int R, int C>
__device__ __forceinline__ void load_stage0_sin(const TileArgs &a, const float2 *sin, unsigned tr, int c, int tl,
                                                float2 (&v)[R])
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, 1>;
    constexpr int r = S::radix(0), NB = R / r, B = TT::B(0), TL = TT::TL;
#pragma unroll
    for (int q = 0; q < R; q++)
        v[q] = make_float2(0.f, 0.f);
    if (tr >= a.ntrans)
        return;
    const int mlim = a.half ? r / 2 : r;
#pragma unroll
    for (int u = 0; u < NB; u++)
#pragma unroll
        for (int m = 0; m < r; m++)
            if (m < mlim)
                v[u * r + m] = sin[(tl + TL * u + m * B) * C + c];
    if (a.conj & 1) {
#pragma unroll
        for (int q = 0; q < R; q++)
            v[q].y = -v[q].y;
    }
}

// W_N^m = exp(-2*pi*i*m/N) for N <= 2^28 a power of two, scale = 2/N; m is
// reduced mod N.  sincospif gets an exactly representable argument: m itself
// when m < 2^24, otherwise the product of the twiddles of m's high and low
// 12-bit parts.
__device__ __forceinline__ float2 fourstep_twiddle(unsigned m, float scale, unsigned mask)
{
    m &= mask;
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

// Shared memory of a tile: the exchange slices ...
template <int L, int R, int C, int Q, int LMAP, int SMAP>
__host__ __device__ constexpr size_t tile_exchange_bytes()
{
    return (Sched<L, R>::NST > 1)
               ? (size_t)C * region_stride<L / Q, C, (LMAP == ACROSS || SMAP == ACROSS)>() * sizeof(float2)
               : 0;
}

constexpr size_t kMaxSmemPerCta = 227 * 1024;

// ... and, for single-CTA column passes where it fits, a four-step twiddle
// region: the per-tile half W_N^(k*C*tile) of every output k (L values, with
// the plan's table tw_lo), or the column powers W_N^(col*off) of the R output
// offsets of each of the C columns (tw_colpow); without it the twiddles come
// from sincospif.
template <int L, int R, int C, int Q, int LMAP, int SMAP>
__host__ __device__ constexpr size_t tile_twr_elems()
{
    return (size_t)L > (size_t)C * R ? (size_t)L : (size_t)C * R;
}

template <int L, int R, int C, int Q, int LMAP, int SMAP>
__host__ __device__ constexpr bool tile_has_thi()
{
    return Q == 1 && LMAP == ACROSS && SMAP == ACROSS &&
           tile_exchange_bytes<L, R, C, Q, LMAP, SMAP>() + tile_twr_elems<L, R, C, Q, LMAP, SMAP>() * sizeof(float2) <=
               kMaxSmemPerCta;
}

template <int L, int R, int C, int Q, int LMAP, int SMAP>
__host__ __device__ constexpr size_t tile_smem_bytes()
{
    return tile_exchange_bytes<L, R, C, Q, LMAP, SMAP>() +
           (tile_has_thi<L, R, C, Q, LMAP, SMAP>() ? tile_twr_elems<L, R, C, Q, LMAP, SMAP>() * sizeof(float2) : 0);
}


// --------------------------------------------------------------- kernel

template <int L, int R, int C, int Q, int LMAP, int SMAP, int s>
__device__ __forceinline__ void run_stages(float2 (&v)[R], int j, int &c, int &tl, float2 *smem,
                                           const float2 *__restrict__ tw)
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, Q>;
    if constexpr (s < S::NST) {
        constexpr int RS = region_stride<TT::LQ, C, (LMAP == ACROSS || SMAP == ACROSS)>();
        stage_write<L, R, Q, s - 1>(smem + c * RS, v, j, tl);
        tile_sync<Q>();
        split_tid<(s == S::NST - 1) ? SMAP : ALONG, C, TT::TL>(threadIdx.x, c, tl);
        stage_read<L, R, Q, s>(smem + c * RS, v, j, tl);
        if (s < S::NST - 1)
            tile_sync<Q>();
        stage_compute<L, R, Q, s>(v, j, tl, tw);
        run_stages<L, R, C, Q, LMAP, SMAP, s + 1>(v, j, c, tl, smem, tw);
    }
}

// Threads of one CTA, and the CTAs per SM the register budget is sized for:
// 16-element tiles are held to 64 registers so that 2048 threads fit.
template <int L, int R, int C, int Q> __host__ __device__ constexpr int tile_threads() { return C * (L / (R * Q)); }
template <int L, int R, int C, int Q> __host__ __device__ constexpr int tile_min_blocks()
{
    return R <= 16 ? (tile_threads<L, R, C, Q>() >= 1024 ? 1 : 1024 / tile_threads<L, R, C, Q>()) : 1;
}

// One tile of C transforms: load, all stages, store.  `tile` selects the
// transforms tile*C .. tile*C + C - 1; ioff / ooff shift the input / output
// base (batches); j is the CTA's rank in its cluster.  COH: load with
// L2-coherent loads (input written earlier in the same launch).
// PRE: the stage-0 registers were loaded by the caller (`pre`, R values).
// C2RS: c2r fix-up prologue through a row staged in shared memory (row
// tiles; the caller checked load_stage0_c2r_rows's conditions).
// EMUL: plain epilogue multiplied by scale * in2[tr*in2_dist + k*in2_stride]
// (the spectral multiply of a convolution, fused into the forward pass).
// TAB: every transform of the tile has its own buffers (in_tab / in2_tab /
// out_tab, distances 0): a tile of C unrelated requests of one size.
template <int L, int R, int C, int Q, int LMAP, int SMAP, bool COH, bool SIN = false, bool PRE = false,
          bool C2RS = false, bool EMUL = false, bool TAB = false>
__device__ __forceinline__ void tile_body(const TileArgs &a, unsigned tile, int j, long long ioff, long long ooff,
                                          float2 *smem, const float2 *sin = nullptr, unsigned twy = 0,
                                          const float2 *pre = nullptr)
{
    using S = Sched<L, R>;
    using TT = Tile<L, R, Q>;
    constexpr int TL = TT::TL, NST = S::NST;
    constexpr int RS = region_stride<TT::LQ, C, (LMAP == ACROSS || SMAP == ACROSS)>();
    static_assert(NST > 1 || LMAP == SMAP, "single-stage tiles cannot change the thread map");
    static_assert(NST > 1 || Q == 1, "single-stage tiles are not split over a cluster");

    const float2 *in = a.in + ioff;
    const float2 *in2 = a.in2 ? a.in2 + ((a.in2_bcast & 1) ? 0 : ioff) : nullptr;
    float2 *out = a.out + ooff;
    static_assert(!TAB || (Q == 1 && LMAP == ALONG && SMAP == ALONG), "per-transform buffers: row tiles");
    const unsigned tile0 = tile * C;

    static_assert(tile_smem_bytes<L, R, C, Q, LMAP, SMAP>() <= kMaxSmemPerCta, "tile exceeds shared memory");
    float2 v[R];
    int c, tl;
    split_tid<LMAP, C, TL>(threadIdx.x, c, tl);
    if constexpr (PRE) {
#pragma unroll
        for (int q = 0; q < R; q++)
            v[q] = pre[q];
    } else if constexpr (SIN) {
        static_assert(Q == 1 && LMAP == ACROSS, "staged inputs are column tiles");
        load_stage0_sin<L, R, C>(a, sin, tile0 + c, c, tl, v);
    } else if constexpr (C2RS) {
        static_assert(LMAP == ALONG && Q == 1 && NST > 1, "staged c2r rows need a row tile with an exchange");
        load_stage0_c2r_rows<L, R, COH>(a, in, in2, tile0 + c, tl, smem + c * RS, v);
        __syncthreads();  // the exchange slices are free again
    } else if constexpr (TAB) {
        const unsigned t = tile0 + c;
        const bool ok = t < a.ntrans;
        load_stage0<L, R, Q, LMAP, COH>(a, ok ? a.in_tab[t] : in, (ok && a.in2_tab) ? a.in2_tab[t] : in2, t, j, tl,
                                        v);
    } else {
        load_stage0<L, R, Q, LMAP, COH>(a, in, in2, tile0 + c, j, tl, v);
    }
    // The four-step twiddle region, and this thread's column-power base, are
    // computed while the stage-0 loads are in flight (the epilogue reads the
    // region after the exchanges' barriers).
    float2 wbase = make_float2(1.f, 0.f);
    if constexpr (tile_has_thi<L, R, C, Q, LMAP, SMAP>()) {
        if (a.epilogue == EPI_TWIDDLE && a.tw_colpow && !a.tw_by_y) {
            int cl, tll;  // the thread's transform and position in the last stage
            split_tid<SMAP, C, TL>(threadIdx.x, cl, tll);
            wbase = fourstep_twiddle((unsigned)(j * TT::B(NST - 1) + tll) * (tile0 + cl), a.tw_scale, a.tw_mask);
        }
    }
    if constexpr (tile_has_thi<L, R, C, Q, LMAP, SMAP>()) {
        float2 *thi = smem + tile_exchange_bytes<L, R, C, Q, LMAP, SMAP>() / sizeof(float2);
        if (a.epilogue == EPI_TWIDDLE && a.tw_by_y) {
            // W_N^(k*row) for every output k, the same for all columns
            for (int k = threadIdx.x; k < L; k += tile_threads<L, R, C, Q>())
                thi[k] = fourstep_twiddle((unsigned)k * twy, a.tw_scale, a.tw_mask);
            if constexpr (NST == 1)
                __syncthreads();
        } else if (a.epilogue == EPI_TWIDDLE && a.tw_colpow) {
            // W_N^(col*off_i), col = tile*C + c, for the last stage's output
            // offsets off_i = TL*u + m*BL of register i = u*rl + m
            constexpr int rl = S::radix(NST - 1), BL = TT::B(NST - 1);
            for (int idx = threadIdx.x; idx < C * R; idx += tile_threads<L, R, C, Q>()) {
                const int cc = idx % C, i = idx / C;  // [i][c]: neighbouring columns in neighbouring banks
                const unsigned off = (unsigned)(TL * (i / rl) + (i % rl) * BL);
                thi[idx] = fourstep_twiddle((tile0 + cc) * off, a.tw_scale, a.tw_mask);
            }
            if constexpr (NST == 1)
                __syncthreads();
        } else if (a.epilogue == EPI_TWIDDLE && a.tw_lo) {
            // Four-step twiddle, per-tile half: W_N^(k*C*tile) for every output k
            // (the per-column half W_N^(k*c) comes from the plan's table tw_lo).
            for (int k = threadIdx.x; k < L; k += tile_threads<L, R, C, Q>())
                thi[k] = fourstep_twiddle((unsigned)k * (unsigned)(C * tile), a.tw_scale, a.tw_mask);
            if constexpr (NST == 1)
                __syncthreads();
        }
    }
    stage_compute<L, R, Q, 0>(v, j, tl, a.tw);
    run_stages<L, R, C, Q, LMAP, SMAP, 1>(v, j, c, tl, smem, a.tw);
    // No CTA of the cluster may leave while others still read its slice.
    if constexpr (Q > 1)
        cg::this_cluster().barrier_arrive();

    // Last stage: register u*rl + m holds output p = j*B + tl + TL*u + m*Q*B.
    constexpr int rl = S::radix(NST - 1), NBL = R / rl, BL = TT::B(NST - 1);
    const unsigned tr = tile0 + c;
    const bool valid = tr < a.ntrans;
    const long long obase = (long long)tr * a.out_dist;
    const int p0 = j * BL + tl;
    if constexpr (TAB) {
        if (valid)
            out = a.out_tab[tr];
    }

    if (a.epilogue == EPI_R2C || a.epilogue == EPI_R2C_FULL) {
        // Z[k] and Z[L-k] sit in different threads (and CTAs): scatter the
        // outputs to their owners' slices, then every CTA resolves its own
        // range of k, reading Z[L-k] wherever it lives.
        constexpr int M = L, LQ = TT::LQ;
        const bool full = a.epilogue == EPI_R2C_FULL;
        if constexpr (NST > 1) {
            float2 *region = smem + c * RS;
            if constexpr (Q > 1)
                cg::this_cluster().barrier_wait();
            else
                __syncthreads();
#pragma unroll
            for (int u = 0; u < NBL; u++)
#pragma unroll
                for (int m = 0; m < rl; m++) {
                    const int pos = p0 + TL * u + m * Q * BL;
                    const int owner = pos / LQ;
                    float2 *dst = Q > 1 ? cg::this_cluster().map_shared_rank(region, owner) : region;
                    dst[padpos(pos - owner * LQ)] = v[u * rl + m];
                }
            tile_sync<Q>();
            if (Q == 1 && valid) {
                // Bins in pairs: Z[k] and Z[M-k] give X[k] = lo and, by the
                // symmetry of a real input's spectrum, X[M-k] = conj(hi) (and
                // X[M+k] = hi, X[2M-k] = conj(lo) for the full output), so a
                // thread resolves k < M/2 and reads each value once.
                const long long os = a.out_stride;
#pragma unroll
                for (int q = 0; q < R / 2; q++) {
                    const int k = tl + TL * q;
                    const float2 zk = region[padpos(k)];
                    if (k == 0) {
                        out[obase] = make_float2(zk.x + zk.y, 0.f);
                        out[obase + (long long)M * os] = make_float2(zk.x - zk.y, 0.f);
                        const float2 zh = region[padpos(M / 2)];  // the middle bin pairs with itself
                        float2 lo, hi;
                        r2c_bins(zh, zh, __ldg(&a.rtw[M / 2]), lo, hi);
                        out[obase + (long long)(M / 2) * os] = lo;
                        if (full)
                            out[obase + (long long)(M / 2 + M) * os] = hi;
                    } else {
                        float2 lo, hi;
                        r2c_bins(zk, region[padpos(M - k)], __ldg(&a.rtw[k]), lo, hi);
                        out[obase + (long long)k * os] = lo;
                        out[obase + (long long)(M - k) * os] = cconj(hi);
                        if (full) {
                            out[obase + (long long)(k + M) * os] = hi;
                            out[obase + (long long)(2 * M - k) * os] = cconj(lo);
                        }
                    }
                }
            } else if (valid) {
#pragma unroll
                for (int q = 0; q < R; q++) {
                    const int kl = tl + TL * q;  // local position in this CTA's slice
                    const int k = j * LQ + kl;
                    const float2 zk = region[padpos(kl)];
                    if (k == 0) {
                        out[obase] = make_float2(zk.x + zk.y, 0.f);
                        out[obase + (long long)M * a.out_stride] = make_float2(zk.x - zk.y, 0.f);
                    } else {
                        const int mk = M - k, mo = mk / LQ;
                        const float2 *src = Q > 1 ? cg::this_cluster().map_shared_rank(region, mo) : region;
                        float2 lo, hi;
                        r2c_bins(zk, src[padpos(mk - mo * LQ)], __ldg(&a.rtw[k]), lo, hi);
                        out[obase + (long long)k * a.out_stride] = lo;
                        if (full)
                            out[obase + (long long)(k + M) * a.out_stride] = hi;
                    }
                }
            }
            if constexpr (Q > 1)
                cg::this_cluster().sync();  // slices stay alive until every CTA has read them
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

    if constexpr (LMAP == ALONG && Q == 1 && NST > 1) {
        // A dead intermediate: every thread has read its inputs (the stage
        // exchanges' barriers lie between), so the tile's input lines leave L2
        // without being written back.  Rows of L points at in_dist, 128-byte
        // aligned (the planner sets the flag only then).
        if (a.l2 & L2_DISCARD_IN) {
            constexpr int LINES = L / 16;  // 128-byte lines per row
            for (int idx = threadIdx.x; idx < C * LINES; idx += tile_threads<L, R, C, Q>()) {
                const unsigned t = tile0 + idx / LINES;
                if (t < a.ntrans) {
                    const float2 *line = in + (long long)t * a.in_dist + 16 * (idx % LINES);
                    asm volatile("discard.global.L2 [%0], 128;" ::"l"(line) : "memory");
                }
            }
        }
    }
    if constexpr (LMAP == ACROSS && Q == 1 && NST > 1 && C * 8 >= 128) {
        // The same for a column tile over a dead intermediate: its input is L
        // row segments of C neighbouring columns (in_dist 1), C * 8 / 128
        // lines each, 128-byte aligned (the planner sets the flag only then);
        // lines that start past the last column are not the tile's.
        if (a.l2 & L2_DISCARD_IN) {
            constexpr int LPR = C * 8 / 128;
            for (int idx = threadIdx.x; idx < L * LPR; idx += tile_threads<L, R, C, Q>()) {
                const unsigned col = tile0 + 16 * (idx % LPR);
                if (col < a.ntrans) {
                    const float2 *line = in + col + (long long)(idx / LPR) * a.in_stride;
                    asm volatile("discard.global.L2 [%0], 128;" ::"l"(line) : "memory");
                }
            }
        }
    }
    const int l2st = a.l2 & (L2_STORE_LAST | L2_STORE_FIRST);
    // every store carries an L2 policy (evict-normal unless the pass asks
    // for another): one instruction form whatever the pass, no branch per
    // store (measured: 2^24 136.2 -> 130-131 us, 4096^2 c2c 131.4 -> 125.8 us
    // against plain stores beside hinted ones)
    const unsigned long long stpol =
        (l2st & L2_STORE_LAST) ? l2_evict_last() : (l2st ? l2_evict_first() : l2_evict_normal());
    if (valid) {
        const long long sst = (SMAP == ALONG) ? 1 : a.out_stride;
        float2 *o0 = out + obase + (long long)p0 * sst;
        if (a.epilogue == EPI_TWIDDLE) {
            // W_N^(k*n) for output k of column n = tile*C + c: the column-power
            // base W_N^(p0*n) (wbase) times the region's W_N^(n*off) (filled
            // while the stage-0 loads were in flight, after the exchange slices)
            float2 *thi = smem + tile_exchange_bytes<L, R, C, Q, LMAP, SMAP>() / sizeof(float2);
#pragma unroll
            for (int u = 0; u < NBL; u++)
#pragma unroll
                for (int m = 0; m < rl; m++) {
                    const int off = TL * u + m * Q * BL;
                    const int k = p0 + off;
                    float2 w;
                    if constexpr (tile_has_thi<L, R, C, Q, LMAP, SMAP>()) {
                        if (a.tw_by_y)
                            w = thi[k];
                        else if (a.tw_colpow)
                            w = cmul(wbase, thi[(u * rl + m) * C + c]);
                        else if (a.tw_lo)
                            w = cmul(__ldg(&a.tw_lo[k * C + c]), thi[k]);
                        else
                            w = fourstep_twiddle((unsigned)k * tr, a.tw_scale, a.tw_mask);
                    } else {
                        w = fourstep_twiddle((unsigned)k * (a.tw_by_y ? twy : tr), a.tw_scale, a.tw_mask);
                    }
                    float2 y = cmul(v[u * rl + m], w);
                    if (a.conj & 2)
                        y.y = -y.y;
                    st_policy(&o0[(long long)off * sst], y, stpol);
                }
        } else {
            const float sg = (a.conj & 2) ? -1.f : 1.f;
#pragma unroll
            for (int u = 0; u < NBL; u++)
#pragma unroll
                for (int m = 0; m < rl; m++) {
                    const int off = TL * u + m * Q * BL;
                    float2 y = v[u * rl + m];
                    if constexpr (EMUL)
                        y = cscale(cmul(y, __ldg(&a.in2[(long long)tr * a.in2_dist + (long long)(p0 + off) * a.in2_stride])),
                                   a.scale);
                    st_policy(&o0[(long long)off * sst], make_float2(y.x, sg * y.y), stpol);
                }
        }
    }
    if constexpr (Q > 1)
        cg::this_cluster().barrier_wait();
}

template <int L, int R, int C, int Q, int LMAP, int SMAP>
__global__ void __launch_bounds__(tile_threads<L, R, C, Q>(), tile_min_blocks<L, R, C, Q>()) tile_fft(const TileArgs a)
{
    extern __shared__ float2 smem[];
    long long ioff, ooff;
    if (a.ysplit) {
        const unsigned g = blockIdx.y % a.ysplit, b = blockIdx.y / a.ysplit;
        ioff = (long long)g * a.in_batch + (long long)b * a.in_batch2;
        ooff = (long long)g * a.out_batch + (long long)b * a.out_batch2;
    } else {
        ioff = (long long)blockIdx.y * a.in_batch;
        ooff = (long long)blockIdx.y * a.out_batch;
    }
    int j = 0;
    unsigned tile = blockIdx.x;
    if constexpr (Q > 1) {
        j = (int)cg::this_cluster().block_rank();
        tile = blockIdx.x / Q;
    }
    tile_body<L, R, C, Q, LMAP, SMAP, false>(a, tile, j, ioff, ooff, smem, nullptr, blockIdx.y);
}

// Row tile whose c2r fix-up prologue stages each row in shared memory
// (load_stage0_c2r_rows); one CTA per tile as tile_fft.
template <int L, int R, int C>
__global__ void __launch_bounds__(tile_threads<L, R, C, 1>(), tile_min_blocks<L, R, C, 1>())
    tile_fft_c2r_rows(const TileArgs a)
{
    extern __shared__ float2 smem[];
    long long ioff, ooff;
    if (a.ysplit) {
        const unsigned g = blockIdx.y % a.ysplit, b = blockIdx.y / a.ysplit;
        ioff = (long long)g * a.in_batch + (long long)b * a.in_batch2;
        ooff = (long long)g * a.out_batch + (long long)b * a.out_batch2;
    } else {
        ioff = (long long)blockIdx.y * a.in_batch;
        ooff = (long long)blockIdx.y * a.out_batch;
    }
    tile_body<L, R, C, 1, ALONG, ALONG, false, false, false, true>(a, blockIdx.x, 0, ioff, ooff, smem);
}

// The staged-c2r variant of a row tile, or null where there is none.
template <int L, int R, int C, int Q> constexpr const void *tile_c2r_rows_fn()
{
    if constexpr (Q == 1 && Sched<L, R>::NST > 1)
        return (const void *)&tile_fft_c2r_rows<L, R, C>;
    else
        return nullptr;
}

}  // namespace mgb
