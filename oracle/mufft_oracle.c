/*
 * mufft_oracle.c -- CPU restatement of muFFT's scalar FFT / convolution path.
 *
 * TEST INFRASTRUCTURE ONLY (see mufft_oracle.h).  Compiled with
 * -ffp-contract=off so every complex multiply rounds the way the reference's
 * portable C kernels round on x86-64.
 *
 * What is restated, and from where in the reference:
 *   twiddle tables ........ fft.c:101-134  exp(i*pi*dir*k/p) in FP64, rounded to
 *                           float; block p at index p (p >= 4), p=2 block at 1..2
 *   planner ............... fft.c:217-256 (1D rules), fft.c:258-287 (vertical
 *                           rules), fft.c:325-435 (first rule that fits wins)
 *   Stockham passes ....... kernel.c:84-453 (1D) and kernel.c:455-738 (vertical):
 *                           a radix-R pass is log2(R) fused radix-2 DIT
 *                           sub-stages; written here once, generically
 *   real <-> complex ...... kernel.c:36-82 (resolves), fft.c:441-455 (twiddles)
 *   executors ............. fft.c:811-989
 *   convolution ........... fft.c:565-624, fft.c:794-809, kernel.c:22-34
 */
#include "mufft_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Public flag values (fft.h:44-65, :131-150). */
#define OR_FORWARD (-1)
#define OR_INVERSE (1)
#define OR_FLAG_FULL_R2C (1u << 16)
#define OR_FLAG_ZERO_PAD_UPPER_HALF (1u << 17)
#define OR_CONV_STEREO 1u
#define OR_CONV_ZP_FIRST (1u << 2)
#define OR_CONV_ZP_SECOND (1u << 3)
#define OR_PAD_SAMPLES 4u /* fft_internal.h:203 */

typedef struct { float re, im; } ocf;

static inline ocf ocf_make(float re, float im) { ocf r = { re, im }; return r; }
static inline ocf ocf_add(ocf a, ocf b) { return ocf_make(a.re + b.re, a.im + b.im); }
static inline ocf ocf_sub(ocf a, ocf b) { return ocf_make(a.re - b.re, a.im - b.im); }
static inline ocf ocf_mul(ocf a, ocf b)
{
    return ocf_make(a.re * b.re - a.im * b.im, a.re * b.im + b.re * a.im);
}
static inline ocf ocf_scale(float s, ocf a) { return ocf_make(a.re * s, a.im * s); }
static inline ocf ocf_conj(ocf a) { return ocf_make(a.re, -a.im); }

static int is_pow2(unsigned n) { return n != 0 && (n & (n - 1)) == 0; }

/* ---------------------------------------------------------------- twiddles */

/* exp(i*pi*dir*k/p) with the phase formed exactly as fft.c:104 does. */
static ocf twiddle_fp64(int dir, int k, int p)
{
    double phase = (M_PI * dir * k) / p;
    return ocf_make((float)cos(phase), (float)sin(phase));
}

/* Index of the block holding the twiddles of sub-transform size p. */
static unsigned tw_block(unsigned p) { return p >= 4 ? p : (p == 2 ? 1 : 0); }

static ocf *make_twiddles(unsigned N, int dir)
{
    unsigned n = N < 4 ? 4 : N;
    ocf *t = calloc(n, sizeof(ocf));
    if (!t)
        return NULL;
    for (unsigned p = 1; p < N; p <<= 1)
        for (unsigned k = 0; k < p; k++)
            t[tw_block(p) + k] = twiddle_fp64(dir, (int)k, (int)p);
    return t;
}

/* i*dir*exp(i*pi*dir*k/M), the real<->complex fix-up twiddles. */
static ocf *make_r2c_twiddles(int dir, unsigned M)
{
    ocf *t = calloc(M ? M : 1, sizeof(ocf));
    if (!t)
        return NULL;
    for (unsigned k = 0; k < M; k++)
        t[k] = ocf_mul(ocf_make(0.0f, (float)dir), twiddle_fp64(dir, (int)k, (int)M));
    return t;
}

/* ----------------------------------------------------------------- planner */

enum { DIR_ANY = 0, DIR_FWD = 1, DIR_INV = 2 };
enum { ZP_ANY = 0, ZP_NO = 1, ZP_YES = 2 };

typedef struct
{
    unsigned radix;
    unsigned fixed_p;  /* nonzero: usable only at this p */
    unsigned min_p;    /* otherwise: usable for p >= min_p */
    int dir;
    int zp;
} rule;

typedef struct
{
    unsigned radix;
    unsigned p;
    int half;   /* first pass of a zero-padded transform: upper half is zero */
} ostep;

/* The portable-C rows of the 1D table, in table order (fft.c:217-256). */
static const rule rules_1d[] = {
    { 8, 1, 0, DIR_FWD, ZP_NO },  { 4, 1, 0, DIR_FWD, ZP_NO },  { 2, 1, 0, DIR_ANY, ZP_NO },
    { 8, 1, 0, DIR_FWD, ZP_YES }, { 4, 1, 0, DIR_FWD, ZP_YES }, { 2, 1, 0, DIR_ANY, ZP_YES },
    { 2, 2, 0, DIR_FWD, ZP_ANY },
    { 8, 1, 0, DIR_INV, ZP_ANY }, { 4, 1, 0, DIR_INV, ZP_ANY }, { 2, 2, 0, DIR_INV, ZP_ANY },
    { 8, 0, 8, DIR_ANY, ZP_ANY }, { 4, 0, 4, DIR_ANY, ZP_ANY }, { 2, 0, 4, DIR_ANY, ZP_ANY },
};

/* The portable-C rows of the vertical table (fft.c:258-287). */
static const rule rules_2d[] = {
    { 8, 1, 0, DIR_FWD, ZP_ANY }, { 4, 1, 0, DIR_FWD, ZP_ANY }, { 2, 1, 0, DIR_ANY, ZP_ANY },
    { 8, 1, 0, DIR_INV, ZP_ANY }, { 4, 1, 0, DIR_INV, ZP_ANY },
    { 8, 0, 8, DIR_ANY, ZP_ANY }, { 4, 0, 4, DIR_ANY, ZP_ANY }, { 2, 0, 2, DIR_ANY, ZP_ANY },
};

static int rule_fits(const rule *r, unsigned remaining, unsigned N, unsigned p, int dir, int zp)
{
    if (remaining % r->radix != 0 || N < r->radix)
        return 0;
    if (r->dir == DIR_FWD && dir != OR_FORWARD)
        return 0;
    if (r->dir == DIR_INV && dir != OR_INVERSE)
        return 0;
    if (r->zp == ZP_NO && zp)
        return 0;
    if (r->zp == ZP_YES && !zp)
        return 0;
    return r->fixed_p ? (p == r->fixed_p) : (p >= r->min_p);
}

/* Greedy decomposition: at each p take the first rule that fits. */
static ostep *plan_steps(unsigned N, int dir, int zp, int vertical, unsigned *count)
{
    const rule *rules = vertical ? rules_2d : rules_1d;
    unsigned nrules = vertical ? sizeof(rules_2d) / sizeof(rules_2d[0])
                               : sizeof(rules_1d) / sizeof(rules_1d[0]);
    ostep *steps = calloc(32, sizeof(ostep));
    unsigned n = 0, remaining = N, p = 1;
    if (!steps)
        return NULL;
    while (remaining > 1)
    {
        unsigned i;
        for (i = 0; i < nrules; i++)
            if (rule_fits(&rules[i], remaining, N, p, dir, zp))
                break;
        if (i == nrules || n == 32)
        {
            free(steps);
            return NULL;
        }
        steps[n].radix = rules[i].radix;
        steps[n].p = p;
        steps[n].half = (rules[i].zp == ZP_YES);
        n++;
        remaining /= rules[i].radix;
        p *= rules[i].radix;
    }
    *count = n;
    return steps;
}

/* ------------------------------------------------------------------ passes */

/*
 * One radix-R Stockham pass over one line of N points (input/output strides
 * in elements).  The R inputs of butterfly i sit at i + m*N/R; they are
 * combined by log2(R) radix-2 DIT sub-stages.  Sub-stage s merges pairs of
 * length-L partial transforms (L = 2^s) into length 2L ones using the
 * twiddles of sub-transform size p*L at offset k + q*p, and the result lands
 * at (i - k)*R + k + q*p.
 *
 * The reference's p = 1 kernels skip multiplications by the exact unit
 * twiddle; this is mirrored (the first vertical radix-8 pass also skips the
 * q = 0 factor of its last sub-stage, kernel.c:650-653) so that even signed
 * zeros agree.
 */
static void stockham_pass(ocf *out, size_t os, const ocf *in, size_t is, const ocf *tw,
                          unsigned radix, unsigned p, unsigned N, int half, int vertical)
{
    unsigned nb = N / radix;
    for (unsigned i = 0; i < nb; i++)
    {
        unsigned k = i & (p - 1);
        ocf v[8], w[8];
        int zero_hi = half;
        for (unsigned m = 0; m < radix; m++)
            v[m] = (half && m >= radix / 2) ? ocf_make(0.0f, 0.0f) : in[(size_t)(i + m * nb) * is];

        for (unsigned L = 1; L < radix; L <<= 1)
        {
            unsigned pairs = radix / (2 * L);
            const ocf *blk = tw + tw_block(p * L);
            for (unsigned j = 0; j < pairs; j++)
            {
                for (unsigned q = 0; q < L; q++)
                {
                    ocf u = v[j * L + q];
                    ocf t = v[(j + pairs) * L + q];
                    if (zero_hi)
                    {
                        w[2 * j * L + q] = u;
                        w[2 * j * L + L + q] = u;
                        continue;
                    }
                    int mul;
                    if (p > 1)
                        mul = 1;
                    else if (L == 1)
                        mul = 0;
                    else if (L == 2)
                        mul = (q > 0);
                    else
                        mul = (q > 0) || !vertical;
                    if (mul)
                        t = ocf_mul(t, blk[k + q * p]);
                    w[2 * j * L + q] = ocf_add(u, t);
                    w[2 * j * L + L + q] = ocf_sub(u, t);
                }
            }
            zero_hi = 0;
            memcpy(v, w, radix * sizeof(ocf));
        }

        unsigned j0 = (i - k) * radix + k;
        for (unsigned q = 0; q < radix; q++)
            out[(size_t)(j0 + q * p) * os] = v[q];
    }
}

/* Run all steps of one line; the last write lands in `out`. */
static void run_line(const ostep *steps, unsigned nsteps, const ocf *tw, unsigned N,
                     ocf *out, size_t os, const ocf *in, size_t is, ocf *scratch /* 2*N */,
                     int vertical)
{
    const ocf *cur = in;
    size_t cs = is;
    for (unsigned s = 0; s < nsteps; s++)
    {
        ocf *dst;
        size_t ds;
        if (s + 1 == nsteps)
        {
            dst = out;
            ds = os;
        }
        else
        {
            dst = scratch + (s & 1) * N;
            ds = 1;
        }
        stockham_pass(dst, ds, cur, cs, tw, steps[s].radix, steps[s].p, N, steps[s].half, vertical);
        cur = dst;
        cs = ds;
    }
}

/* kernel.c:36-45 */
static void resolve_c2r(ocf *out, const ocf *in, const ocf *tw, unsigned M)
{
    for (unsigned i = 0; i < M; i++)
    {
        ocf a = in[i];
        ocf b = ocf_conj(in[M - i]);
        out[i] = ocf_add(ocf_add(a, b), ocf_mul(ocf_sub(a, b), tw[i]));
    }
}

/* kernel.c:47-82 */
static void resolve_r2c(ocf *out, const ocf *in, const ocf *tw, unsigned M, int full)
{
    ocf fe0 = ocf_make(in[0].re, 0.0f);
    ocf fo0 = ocf_make(in[0].im, 0.0f);
    out[0] = ocf_add(fe0, fo0);
    out[M] = ocf_sub(fe0, fo0);
    for (unsigned i = 1; i < M; i++)
    {
        ocf a = in[i];
        ocf b = ocf_conj(in[M - i]);
        ocf fe = ocf_add(a, b);
        ocf fo = ocf_mul(tw[i], ocf_sub(a, b));
        out[i] = ocf_scale(0.5f, ocf_add(fe, fo));
        if (full)
            out[i + M] = ocf_scale(0.5f, ocf_sub(fe, fo));
    }
}

/* kernel.c:22-34 */
void oracle_convolve(void *output, const void *a_, const void *b_, float normalization, unsigned samples)
{
    ocf *o = output;
    const ocf *a = a_, *b = b_;
    for (unsigned i = 0; i < samples; i++)
        o[i] = ocf_scale(normalization, ocf_mul(a[i], b[i]));
}

/* -------------------------------------------------------------------- 1D */

enum { KIND_C2C = 0, KIND_R2C = 1, KIND_R2C_FULL = 2, KIND_C2R = 3 };

struct oracle_plan_1d
{
    unsigned N;          /* length of the complex transform */
    int kind;
    ostep *steps;
    unsigned nsteps;
    ocf *tw;
    ocf *r2c_tw;
};

oracle_plan_1d *oracle_create_plan_1d_c2c(unsigned N, int direction, unsigned flags)
{
    if (!is_pow2(N) || N == 1)
        return NULL;
    if (direction != OR_FORWARD && direction != OR_INVERSE)
        return NULL;
    oracle_plan_1d *pl = calloc(1, sizeof(*pl));
    if (!pl)
        return NULL;
    pl->N = N;
    pl->kind = KIND_C2C;
    pl->tw = make_twiddles(N, direction);
    pl->steps = plan_steps(N, direction, (flags & OR_FLAG_ZERO_PAD_UPPER_HALF) != 0, 0, &pl->nsteps);
    if (!pl->tw || !pl->steps)
    {
        oracle_free_plan_1d(pl);
        return NULL;
    }
    return pl;
}

oracle_plan_1d *oracle_create_plan_1d_r2c(unsigned N, unsigned flags)
{
    if (!is_pow2(N) || N == 1)
        return NULL;
    oracle_plan_1d *pl = oracle_create_plan_1d_c2c(N / 2, OR_FORWARD, flags);
    if (!pl)
        return NULL;
    pl->kind = (flags & OR_FLAG_FULL_R2C) ? KIND_R2C_FULL : KIND_R2C;
    pl->r2c_tw = make_r2c_twiddles(OR_FORWARD, N / 2);
    if (!pl->r2c_tw)
    {
        oracle_free_plan_1d(pl);
        return NULL;
    }
    return pl;
}

oracle_plan_1d *oracle_create_plan_1d_c2r(unsigned N, unsigned flags)
{
    if (!is_pow2(N) || N == 1)
        return NULL;
    oracle_plan_1d *pl = oracle_create_plan_1d_c2c(N / 2, OR_INVERSE, flags);
    if (!pl)
        return NULL;
    pl->kind = KIND_C2R;
    pl->r2c_tw = make_r2c_twiddles(OR_INVERSE, N / 2);
    if (!pl->r2c_tw)
    {
        oracle_free_plan_1d(pl);
        return NULL;
    }
    return pl;
}

unsigned oracle_plan_1d_steps(const oracle_plan_1d *plan, unsigned *radix, unsigned *p, unsigned max_steps)
{
    unsigned n = plan->nsteps < max_steps ? plan->nsteps : max_steps;
    for (unsigned i = 0; i < n; i++)
    {
        radix[i] = plan->steps[i].radix;
        p[i] = plan->steps[i].p;
    }
    return plan->nsteps;
}

/* scratch: 4*N complex */
static void execute_1d(const oracle_plan_1d *pl, void *output, const void *input, ocf *scratch)
{
    unsigned N = pl->N;
    ocf *line = scratch + 2 * N;
    ocf *resolved = scratch + 3 * N;
    const ocf *src = input;
    if (pl->kind == KIND_C2R)
    {
        resolve_c2r(resolved, input, pl->r2c_tw, N);
        src = resolved;
    }
    if (pl->kind == KIND_R2C || pl->kind == KIND_R2C_FULL)
    {
        run_line(pl->steps, pl->nsteps, pl->tw, N, line, 1, src, 1, scratch, 0);
        resolve_r2c(output, line, pl->r2c_tw, N, pl->kind == KIND_R2C_FULL);
    }
    else
    {
        run_line(pl->steps, pl->nsteps, pl->tw, N, output, 1, src, 1, scratch, 0);
    }
}

void oracle_execute_plan_1d(oracle_plan_1d *plan, void *output, const void *input)
{
    ocf *scratch = malloc((size_t)4 * plan->N * sizeof(ocf));
    if (!scratch)
        return;
    execute_1d(plan, output, input, scratch);
    free(scratch);
}

typedef struct
{
    const oracle_plan_1d *plan;
    char *out;
    const char *in;
    size_t out_stride, in_stride;
    unsigned begin, end;
} many_job;

static void *many_worker(void *arg)
{
    many_job *j = arg;
    ocf *scratch = malloc((size_t)4 * j->plan->N * sizeof(ocf));
    if (!scratch)
        return NULL;
    for (unsigned i = j->begin; i < j->end; i++)
        execute_1d(j->plan, j->out + i * j->out_stride, j->in + i * j->in_stride, scratch);
    free(scratch);
    return NULL;
}

void oracle_execute_plan_1d_many(oracle_plan_1d *plan, void *output, const void *input,
                                 unsigned count, size_t out_stride, size_t in_stride,
                                 unsigned nthreads)
{
    if (nthreads < 1)
        nthreads = 1;
    if (nthreads > count)
        nthreads = count ? count : 1;
    pthread_t th[256];
    many_job jobs[256];
    if (nthreads > 256)
        nthreads = 256;
    for (unsigned t = 0; t < nthreads; t++)
    {
        jobs[t].plan = plan;
        jobs[t].out = output;
        jobs[t].in = input;
        jobs[t].out_stride = out_stride;
        jobs[t].in_stride = in_stride;
        jobs[t].begin = (unsigned)((unsigned long long)count * t / nthreads);
        jobs[t].end = (unsigned)((unsigned long long)count * (t + 1) / nthreads);
    }
    for (unsigned t = 1; t < nthreads; t++)
        if (pthread_create(&th[t], NULL, many_worker, &jobs[t]) != 0)
            many_worker(&jobs[t]), th[t] = 0;
    many_worker(&jobs[0]);
    for (unsigned t = 1; t < nthreads; t++)
        if (th[t])
            pthread_join(th[t], NULL);
}

void oracle_free_plan_1d(oracle_plan_1d *plan)
{
    if (!plan)
        return;
    free(plan->steps);
    free(plan->tw);
    free(plan->r2c_tw);
    free(plan);
}

/* ------------------------------------------------------------------ conv */

struct oracle_plan_conv
{
    oracle_plan_1d *in_plan[2];
    oracle_plan_1d *out_plan;
    size_t block_size;
    float normalization;
    unsigned multiply_n;
};

oracle_plan_conv *oracle_create_plan_conv(unsigned N, unsigned flags, unsigned method)
{
    if (!is_pow2(N) || N == 1)
        return NULL;
    oracle_plan_conv *c = calloc(1, sizeof(*c));
    if (!c)
        return NULL;
    unsigned zp0 = (method & OR_CONV_ZP_FIRST) ? OR_FLAG_ZERO_PAD_UPPER_HALF : 0;
    unsigned zp1 = (method & OR_CONV_ZP_SECOND) ? OR_FLAG_ZERO_PAD_UPPER_HALF : 0;
    if ((method & 1u) == OR_CONV_STEREO)
    {
        c->block_size = (size_t)N * sizeof(ocf);
        c->in_plan[0] = oracle_create_plan_1d_c2c(N, OR_FORWARD, flags | zp0);
        c->in_plan[1] = oracle_create_plan_1d_r2c(N, flags | zp1 | OR_FLAG_FULL_R2C);
        c->out_plan = oracle_create_plan_1d_c2c(N, OR_INVERSE, flags);
        c->multiply_n = N;
    }
    else
    {
        c->block_size = (size_t)(N / 2 + OR_PAD_SAMPLES) * sizeof(ocf);
        c->in_plan[0] = oracle_create_plan_1d_r2c(N, flags | zp0);
        c->in_plan[1] = oracle_create_plan_1d_r2c(N, flags | zp1);
        c->out_plan = oracle_create_plan_1d_c2r(N, flags);
        c->multiply_n = N / 2 + 1;
    }
    c->normalization = 1.0f / N;
    if (!c->in_plan[0] || !c->in_plan[1] || !c->out_plan)
    {
        oracle_free_plan_conv(c);
        return NULL;
    }
    return c;
}

void oracle_execute_conv_input(oracle_plan_conv *plan, unsigned block, void *output, const void *input)
{
    oracle_execute_plan_1d(plan->in_plan[block ? 1 : 0], output, input);
}

size_t oracle_conv_get_transformed_block_size(oracle_plan_conv *plan)
{
    return plan->block_size;
}

void oracle_execute_conv_output(oracle_plan_conv *plan, void *output, const void *first, const void *second)
{
    ocf *product = calloc(plan->block_size / sizeof(ocf) + 1, sizeof(ocf));
    if (!product)
        return;
    oracle_convolve(product, first, second, plan->normalization, plan->multiply_n);
    oracle_execute_plan_1d(plan->out_plan, output, product);
    free(product);
}

void oracle_free_plan_conv(oracle_plan_conv *plan)
{
    if (!plan)
        return;
    oracle_free_plan_1d(plan->in_plan[0]);
    oracle_free_plan_1d(plan->in_plan[1]);
    oracle_free_plan_1d(plan->out_plan);
    free(plan);
}

/* -------------------------------------------------------------------- 2D */

struct oracle_plan_2d
{
    unsigned Nx, Ny;         /* Nx: complex row length of the inner transform */
    int kind;
    unsigned vertical_nx;    /* columns touched by the vertical pass */
    ostep *steps_x, *steps_y;
    unsigned nsx, nsy;
    ocf *tw_x, *tw_y, *r2c_tw;
};

oracle_plan_2d *oracle_create_plan_2d_c2c(unsigned Nx, unsigned Ny, int direction, unsigned flags)
{
    if (!is_pow2(Nx) || !is_pow2(Ny) || Nx == 1 || Ny == 1)
        return NULL;
    if (direction != OR_FORWARD && direction != OR_INVERSE)
        return NULL;
    oracle_plan_2d *pl = calloc(1, sizeof(*pl));
    if (!pl)
        return NULL;
    pl->Nx = Nx;
    pl->Ny = Ny;
    pl->kind = KIND_C2C;
    pl->vertical_nx = Nx;
    pl->tw_x = make_twiddles(Nx, direction);
    pl->tw_y = make_twiddles(Ny, direction);
    pl->steps_x = plan_steps(Nx, direction, (flags & OR_FLAG_ZERO_PAD_UPPER_HALF) != 0, 0, &pl->nsx);
    pl->steps_y = plan_steps(Ny, direction, 0, 1, &pl->nsy);
    if (!pl->tw_x || !pl->tw_y || !pl->steps_x || !pl->steps_y)
    {
        oracle_free_plan_2d(pl);
        return NULL;
    }
    return pl;
}

oracle_plan_2d *oracle_create_plan_2d_r2c(unsigned Nx, unsigned Ny, unsigned flags)
{
    if (!is_pow2(Nx) || !is_pow2(Ny) || Nx == 1 || Ny == 1)
        return NULL;
    oracle_plan_2d *pl = oracle_create_plan_2d_c2c(Nx / 2, Ny, OR_FORWARD, flags);
    if (!pl)
        return NULL;
    pl->kind = (flags & OR_FLAG_FULL_R2C) ? KIND_R2C_FULL : KIND_R2C;
    pl->vertical_nx = (flags & OR_FLAG_FULL_R2C) ? Nx : Nx / 2 + 1;
    pl->r2c_tw = make_r2c_twiddles(OR_FORWARD, Nx / 2);
    if (!pl->r2c_tw)
    {
        oracle_free_plan_2d(pl);
        return NULL;
    }
    return pl;
}

oracle_plan_2d *oracle_create_plan_2d_c2r(unsigned Nx, unsigned Ny, unsigned flags)
{
    if (!is_pow2(Nx) || !is_pow2(Ny) || Nx == 1 || Ny == 1)
        return NULL;
    oracle_plan_2d *pl = oracle_create_plan_2d_c2c(Nx / 2, Ny, OR_INVERSE, flags);
    if (!pl)
        return NULL;
    pl->kind = KIND_C2R;
    pl->vertical_nx = Nx / 2 + 1;
    pl->r2c_tw = make_r2c_twiddles(OR_INVERSE, Nx / 2);
    if (!pl->r2c_tw)
    {
        oracle_free_plan_2d(pl);
        return NULL;
    }
    return pl;
}

/* Vertical transform of `ncols` columns in place on a row-major grid. */
static void columns(const oracle_plan_2d *pl, ocf *grid, size_t stride, unsigned ncols)
{
    unsigned Ny = pl->Ny;
    ocf *col = malloc((size_t)3 * Ny * sizeof(ocf));
    if (!col)
        return;
    for (unsigned x = 0; x < ncols; x++)
    {
        run_line(pl->steps_y, pl->nsy, pl->tw_y, Ny, grid + x, stride, grid + x, stride, col, 1);
    }
    free(col);
}

void oracle_execute_plan_2d(oracle_plan_2d *pl, void *output, const void *input)
{
    unsigned Nx = pl->Nx, Ny = pl->Ny;
    ocf *scratch = malloc((size_t)4 * Nx * sizeof(ocf));
    if (!scratch)
        return;
    if (pl->kind == KIND_C2C)
    {
        ocf *out = output;
        const ocf *in = input;
        for (unsigned y = 0; y < Ny; y++)
            run_line(pl->steps_x, pl->nsx, pl->tw_x, Nx, out + (size_t)y * Nx, 1,
                     in + (size_t)y * Nx, 1, scratch, 0);
        columns(pl, out, Nx, Nx);
    }
    else if (pl->kind == KIND_R2C || pl->kind == KIND_R2C_FULL)
    {
        /* rows: real 2*Nx samples -> Nx complex FFT -> resolve into a row of
         * stride 2*Nx complex (fft.c:939-972) */
        ocf *out = output;
        const ocf *in = input;
        ocf *line = scratch + 2 * Nx;
        for (unsigned y = 0; y < Ny; y++)
        {
            run_line(pl->steps_x, pl->nsx, pl->tw_x, Nx, line, 1, in + (size_t)y * Nx, 1, scratch, 0);
            resolve_r2c(out + (size_t)y * 2 * Nx, line, pl->r2c_tw, Nx, pl->kind == KIND_R2C_FULL);
        }
        columns(pl, out, 2 * (size_t)Nx, pl->vertical_nx);
    }
    else
    {
        /* c2r: columns first on a copy of the input (fft.c:863-916) */
        size_t total = (size_t)Ny * 2 * Nx;
        ocf *grid = malloc(total * sizeof(ocf));
        if (!grid)
        {
            free(scratch);
            return;
        }
        memcpy(grid, input, total * sizeof(ocf));
        columns(pl, grid, 2 * (size_t)Nx, pl->vertical_nx);
        ocf *out = output;
        ocf *line = scratch + 2 * Nx;
        for (unsigned y = 0; y < Ny; y++)
        {
            resolve_c2r(line, grid + (size_t)y * 2 * Nx, pl->r2c_tw, Nx);
            run_line(pl->steps_x, pl->nsx, pl->tw_x, Nx, out + (size_t)y * Nx, 1, line, 1, scratch, 0);
        }
        free(grid);
    }
    free(scratch);
}

void oracle_free_plan_2d(oracle_plan_2d *plan)
{
    if (!plan)
        return;
    free(plan->steps_x);
    free(plan->steps_y);
    free(plan->tw_x);
    free(plan->tw_y);
    free(plan->r2c_tw);
    free(plan);
}

/* ------------------------------------------------------------- FP64 DFT */

void oracle_dft_f64(double *out, const double *in, unsigned N, int direction)
{
    for (unsigned k = 0; k < N; k++)
    {
        double sr = 0.0, si = 0.0;
        for (unsigned n = 0; n < N; n++)
        {
            unsigned long long idx = ((unsigned long long)n * k) % N;
            double ph = 2.0 * M_PI * (double)direction * (double)idx / (double)N;
            double c = cos(ph), s = sin(ph);
            double xr = in[2 * n], xi = in[2 * n + 1];
            sr += xr * c - xi * s;
            si += xr * s + xi * c;
        }
        out[2 * k] = sr;
        out[2 * k + 1] = si;
    }
}
