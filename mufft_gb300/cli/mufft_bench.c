/* muFFT-style command-line benchmark for libmufft_gb300.
 *
 * Same arguments and line layout as the reference's bench.c (bench.c:586-633):
 *   mufft-bench                       1D sweep N = 4 .. 128K, then 2D 4..1024 per side
 *   mufft-bench <iterations> <N>      1D c2c, r2c + c2r, convolution
 *   mufft-bench <iterations> <Nx> <Ny>  2D c2c, r2c, c2r
 * FFTW (the reference's comparator) is not available; instead each line of
 * this library is printed next to the reference library itself when
 * MUFFT_REFERENCE_LIB names its shared object (oracle/build_ref.sh builds one),
 * loaded with dlopen so the two identical APIs do not collide.
 *
 * Lines "muFFT-GB300 ..." go through the reference API (fft.h) on mufft_alloc
 * buffers -- synchronous, host buffers, transfers included, as a muFFT caller
 * sees it; "muFFT-GB300 device ..." lines time the same plan on device
 * buffers (mufft_gb300.h asynchronous execute, kernels only).  Mflops use the
 * reference's estimates (5 N log2 N per complex transform).  Iteration
 * counts of the sweep follow bench.c (400000000 / (N + 16)) capped at 20000.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "fft.h"
#include "mufft_gb300.h"

static double now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* The reference library's entry points, resolved with dlsym. */
struct api {
    void *h;
    mufft_plan_1d *(*c2c)(unsigned, int, unsigned);
    mufft_plan_1d *(*r2c)(unsigned, unsigned);
    mufft_plan_1d *(*c2r)(unsigned, unsigned);
    void (*exec1)(mufft_plan_1d *, void *, const void *);
    void (*free1)(mufft_plan_1d *);
    mufft_plan_2d *(*c2c2)(unsigned, unsigned, int, unsigned);
    mufft_plan_2d *(*r2c2)(unsigned, unsigned, unsigned);
    mufft_plan_2d *(*c2r2)(unsigned, unsigned, unsigned);
    void (*exec2)(mufft_plan_2d *, void *, const void *);
    void (*free2)(mufft_plan_2d *);
    mufft_plan_conv *(*conv)(unsigned, unsigned, unsigned);
    void (*cin)(mufft_plan_conv *, unsigned, void *, const void *);
    void (*cout)(mufft_plan_conv *, void *, const void *, const void *);
    size_t (*cbs)(mufft_plan_conv *);
    void (*cfree)(mufft_plan_conv *);
    void *(*alloc)(size_t);
    void (*mfree)(void *);
};

static struct api gpu_api(void)
{
    struct api a = {0};
    a.c2c = mufft_create_plan_1d_c2c;
    a.r2c = mufft_create_plan_1d_r2c;
    a.c2r = mufft_create_plan_1d_c2r;
    a.exec1 = mufft_execute_plan_1d;
    a.free1 = mufft_free_plan_1d;
    a.c2c2 = mufft_create_plan_2d_c2c;
    a.r2c2 = mufft_create_plan_2d_r2c;
    a.c2r2 = mufft_create_plan_2d_c2r;
    a.exec2 = mufft_execute_plan_2d;
    a.free2 = mufft_free_plan_2d;
    a.conv = mufft_create_plan_conv;
    a.cin = mufft_execute_conv_input;
    a.cout = mufft_execute_conv_output;
    a.cbs = mufft_conv_get_transformed_block_size;
    a.cfree = mufft_free_plan_conv;
    a.alloc = mufft_alloc;
    a.mfree = mufft_free;
    return a;
}

static int ref_api(struct api *a)
{
    const char *path = getenv("MUFFT_REFERENCE_LIB");
    if (!path || !*path)
        return 0;
    memset(a, 0, sizeof(*a));
    a->h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!a->h) {
        fprintf(stderr, "cannot load %s: %s\n", path, dlerror());
        return 0;
    }
#define SYM(f, n) *(void **)(&a->f) = dlsym(a->h, n)
    SYM(c2c, "mufft_create_plan_1d_c2c");
    SYM(r2c, "mufft_create_plan_1d_r2c");
    SYM(c2r, "mufft_create_plan_1d_c2r");
    SYM(exec1, "mufft_execute_plan_1d");
    SYM(free1, "mufft_free_plan_1d");
    SYM(c2c2, "mufft_create_plan_2d_c2c");
    SYM(r2c2, "mufft_create_plan_2d_r2c");
    SYM(c2r2, "mufft_create_plan_2d_c2r");
    SYM(exec2, "mufft_execute_plan_2d");
    SYM(free2, "mufft_free_plan_2d");
    SYM(conv, "mufft_create_plan_conv");
    SYM(cin, "mufft_execute_conv_input");
    SYM(cout, "mufft_execute_conv_output");
    SYM(cbs, "mufft_conv_get_transformed_block_size");
    SYM(cfree, "mufft_free_plan_conv");
    SYM(alloc, "mufft_alloc");
    SYM(mfree, "mufft_free");
#undef SYM
    return a->c2c && a->exec1 && a->alloc && a->mfree && a->conv && a->exec2;
}

static struct api G, R;
static int have_ref;

/* Seeded inputs (a fixed LCG, the same for every library). */
static void fill(float *p, size_t n, unsigned seed)
{
    unsigned s = seed * 2654435761u + 1;
    for (size_t i = 0; i < n; i++) {
        s = s * 1664525u + 1013904223u;
        p[i] = (float)(s >> 8) * (1.0f / 16777216.0f) - 0.5f;
    }
}

static double time_1d(const struct api *a, int kind, unsigned N, unsigned iters)
{
    float *in = a->alloc(2 * (size_t)N * sizeof(float) + 64);
    float *out = a->alloc(2 * (size_t)N * sizeof(float) + 64);
    float *mid = a->alloc(2 * (size_t)N * sizeof(float) + 64);
    double t = -1.0;
    if (!in || !out || !mid) {
        a->mfree(in);
        a->mfree(out);
        a->mfree(mid);
        return t;
    }
    fill(in, 2 * (size_t)N, 1);
    if (kind == 0) {
        mufft_plan_1d *p = a->c2c(N, MUFFT_FORWARD, 0);
        if (p) {
            a->exec1(p, out, in);
            const double t0 = now();
            for (unsigned i = 0; i < iters; i++)
                a->exec1(p, out, in);
            t = now() - t0;
            a->free1(p);
        }
    } else {
        mufft_plan_1d *f = a->r2c(N, kind == 2 ? MUFFT_FLAG_ZERO_PAD_UPPER_HALF : 0);
        mufft_plan_1d *b = a->c2r(N, 0);
        if (f && b) {
            a->exec1(f, mid, in);
            a->exec1(b, out, mid);
            const double t0 = now();
            for (unsigned i = 0; i < iters; i++) {
                a->exec1(f, mid, in);
                a->exec1(b, out, mid);
            }
            t = now() - t0;
        }
        a->free1(f);
        a->free1(b);
    }
    a->mfree(in);
    a->mfree(out);
    a->mfree(mid);
    return t;
}

static double time_conv(const struct api *a, unsigned N, unsigned iters, int stereo)
{
    const unsigned method = (stereo ? MUFFT_CONV_METHOD_FLAG_STEREO_MONO : MUFFT_CONV_METHOD_FLAG_MONO_MONO) |
                            MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST |
                            MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND;
    mufft_plan_conv *p = a->conv(2 * N, 0, method);
    if (!p)
        return -1.0;
    const size_t bs = a->cbs(p);
    float *x = a->alloc(4 * (size_t)N * sizeof(float) + 64);
    float *h = a->alloc(4 * (size_t)N * sizeof(float) + 64);
    float *out = a->alloc(4 * (size_t)N * sizeof(float) + 64);
    void *b0 = a->alloc(bs), *b1 = a->alloc(bs);
    if (!x || !h || !out || !b0 || !b1) {
        a->mfree(x);
        a->mfree(h);
        a->mfree(out);
        a->mfree(b0);
        a->mfree(b1);
        a->cfree(p);
        return -1.0;
    }
    fill(x, 4 * (size_t)N, 2);
    fill(h, 4 * (size_t)N, 3);
    a->cin(p, MUFFT_CONV_BLOCK_SECOND, b1, h);
    a->cin(p, MUFFT_CONV_BLOCK_FIRST, b0, x);
    a->cout(p, out, b0, b1);
    const double t0 = now();
    for (unsigned i = 0; i < iters; i++) {
        a->cin(p, MUFFT_CONV_BLOCK_FIRST, b0, x);
        a->cout(p, out, b0, b1);
    }
    const double t = now() - t0;
    a->mfree(x);
    a->mfree(h);
    a->mfree(out);
    a->mfree(b0);
    a->mfree(b1);
    a->cfree(p);
    return t;
}

static double time_2d(const struct api *a, int kind, unsigned Nx, unsigned Ny, unsigned iters)
{
    const size_t n = (size_t)Nx * Ny;
    float *in = a->alloc(4 * n * sizeof(float) + 64);
    float *out = a->alloc(4 * n * sizeof(float) + 64);
    if (!in || !out) {
        a->mfree(in);
        a->mfree(out);
        return -1.0;
    }
    fill(in, 2 * n, 4);
    mufft_plan_2d *p = kind == 0 ? a->c2c2(Nx, Ny, MUFFT_FORWARD, 0) : kind == 1 ? a->r2c2(Nx, Ny, 0) : a->c2r2(Nx, Ny, 0);
    double t = -1.0;
    if (p) {
        a->exec2(p, out, in);
        const double t0 = now();
        for (unsigned i = 0; i < iters; i++)
            a->exec2(p, out, in);
        t = now() - t0;
        a->free2(p);
    }
    a->mfree(in);
    a->mfree(out);
    return t;
}

/* Kernel-only time of the same c2c plan on device buffers. */
static double time_1d_device(unsigned N, unsigned iters)
{
    void *din = mufft_gb_device_alloc(8 * (size_t)N), *dout = mufft_gb_device_alloc(8 * (size_t)N);
    mufft_plan_1d *p = mufft_create_plan_1d_c2c(N, MUFFT_FORWARD, 0);
    double t = -1.0;
    if (p && din && dout && mufft_gb_execute_plan_1d_async(p, dout, din, NULL) == MUFFT_GB_OK) {
        mufft_gb_device_synchronize();
        const double t0 = now();
        for (unsigned i = 0; i < iters; i++)
            mufft_gb_execute_plan_1d_async(p, dout, din, NULL);
        mufft_gb_device_synchronize();
        t = now() - t0;
    }
    mufft_free_plan_1d(p);
    mufft_gb_device_free(din);
    mufft_gb_device_free(dout);
    return t;
}

static void line1(const char *what, unsigned N, double flops, double t, unsigned iters)
{
    if (t < 0)
        printf("%-28s%06u        (unavailable)\n", what, N);
    else if (flops > 0)
        printf("%-28s%06u %12.3f Mflops %12.3f us iteration\n", what, N, flops * iters / (1e6 * t), 1e6 * t / iters);
    else
        printf("%-28s%06u %12.3f us iteration\n", what, N, 1e6 * t / iters);
}

static void line2(const char *what, unsigned Nx, unsigned Ny, double flops, double t, unsigned iters)
{
    if (t < 0)
        printf("%-28s%04u by %04u,        (unavailable)\n", what, Nx, Ny);
    else
        printf("%-28s%04u by %04u, %12.3f Mflops %12.3f us iteration\n", what, Nx, Ny, flops * iters / (1e6 * t),
               1e6 * t / iters);
}

static void bench_1d(unsigned N, unsigned iters)
{
    const double flops = 5.0 * N * log2((double)N);
    if (have_ref)
        line1("muFFT C2C:", N, flops, time_1d(&R, 0, N, iters), iters);
    line1("muFFT-GB300 C2C:", N, flops, time_1d(&G, 0, N, iters), iters);
    line1("muFFT-GB300 device C2C:", N, flops, time_1d_device(N, iters), iters);
    if (have_ref) {
        line1("muFFT R2C-C2R:", N, flops, time_1d(&R, 1, N, iters), iters);
        line1("muFFT half R2C-C2R:", N, flops, time_1d(&R, 2, N, iters), iters);
    }
    line1("muFFT-GB300 R2C-C2R:", N, flops, time_1d(&G, 1, N, iters), iters);
    line1("muFFT-GB300 half R2C-C2R:", N, flops, time_1d(&G, 2, N, iters), iters);
    if (have_ref) {
        line1("muFFT conv mono:", N, 0, time_conv(&R, N, iters, 0), iters);
        line1("muFFT conv stereo:", N, 0, time_conv(&R, N, iters, 1), iters);
    }
    line1("muFFT-GB300 conv mono:", N, 0, time_conv(&G, N, iters, 0), iters);
    line1("muFFT-GB300 conv stereo:", N, 0, time_conv(&G, N, iters, 1), iters);
    fflush(stdout);
}

static void bench_2d(unsigned Nx, unsigned Ny, unsigned iters, int all_kinds)
{
    const double c2c = 5.0 * Ny * Nx * log2((double)Nx) + 5.0 * Nx * Ny * log2((double)Ny);
    const double half = 0.5 * c2c;
    static const char *names[3][2] = {{"muFFT:", "muFFT-GB300:"}, {"muFFT R2C:", "muFFT-GB300 R2C:"},
                                      {"muFFT C2R:", "muFFT-GB300 C2R:"}};
    for (int k = 0; k < (all_kinds ? 3 : 1); k++) {
        if (have_ref)
            line2(names[k][0], Nx, Ny, k ? half : c2c, time_2d(&R, k, Nx, Ny, iters), iters);
        line2(names[k][1], Nx, Ny, k ? half : c2c, time_2d(&G, k, Nx, Ny, iters), iters);
    }
    fflush(stdout);
}

static unsigned sweep_iters(unsigned long long n)
{
    const unsigned long long it = 400000000ull / (n + 16);
    return (unsigned)(it > 20000 ? 20000 : (it ? it : 1));
}

int main(int argc, char *argv[])
{
    if (argc == 2 || argc > 4) {
        fprintf(stderr, "Usage: %s [iterations] [Nx] [Ny]\n", argv[0]);
        return 1;
    }
    G = gpu_api();
    have_ref = ref_api(&R);
    if (argc == 1) {
        printf("\n1D benchmarks ...\n");
        for (unsigned N = 4; N <= 128 * 1024; N <<= 1)
            bench_1d(N, sweep_iters(N));
        printf("\n2D benchmarks ...\n");
        for (unsigned Ny = 4; Ny <= 1024; Ny <<= 1)
            for (unsigned Nx = 4; Nx <= 1024; Nx <<= 1)
                bench_2d(Nx, Ny, sweep_iters((unsigned long long)Nx * Ny), 0);
    } else if (argc == 3) {
        bench_1d((unsigned)strtoul(argv[2], NULL, 0), (unsigned)strtoul(argv[1], NULL, 0));
    } else {
        bench_2d((unsigned)strtoul(argv[2], NULL, 0), (unsigned)strtoul(argv[3], NULL, 0),
                 (unsigned)strtoul(argv[1], NULL, 0), 1);
    }
    if (mufft_gb_last_error() != MUFFT_GB_OK)
        fprintf(stderr, "last error: %s\n", mufft_gb_last_error_string());
    return 0;
}
