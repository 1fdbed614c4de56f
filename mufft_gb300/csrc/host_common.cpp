// Host-side common parts of libmufft_gb300: errors, kernel registry lookups,
// per-plan options, per-device state and FP64 tables, memory helpers.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "host.h"

namespace mgb {

// ================================================================ errors

thread_local int t_err = 0;
thread_local char t_errmsg[512] = "";

void set_error(int code, const char *fmt, ...)
{
    t_err = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_errmsg, sizeof(t_errmsg), fmt, ap);
    va_end(ap);
}

bool cuda_ok(cudaError_t e, const char *what)
{
    if (e == cudaSuccess)
        return true;
    set_error((int)e, "%s: %s", what, cudaGetErrorString(e));
    return false;
}

DeviceGuard::DeviceGuard(int dev)
{
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        prev = -1;
    }
    if (dev >= 0 && dev != prev)
        cudaSetDevice(dev);
}

DeviceGuard::~DeviceGuard()
{
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
        cudaSetDevice(prev);
}

// ============================================================= registry

const std::vector<TileKernel> &tile_table()
{
    static const std::vector<TileKernel> t = [] {
        std::vector<TileKernel> v;
        register_tiles_along(v);
        register_tiles_across(v);
        register_tiles_transpose(v);
        return v;
    }();
    return t;
}

static const std::vector<TmaTileKernel> &tma_table()
{
    static const std::vector<TmaTileKernel> t = [] {
        std::vector<TmaTileKernel> v;
        register_tiles_tma(v);
        return v;
    }();
    return t;
}

const TmaTileKernel *find_tma(int L, int R, int C, int nbuf)
{
    for (const TmaTileKernel &k : tma_table())
        if (k.L == L && k.R == R && k.C == C && k.nbuf == nbuf)
            return &k;
    return nullptr;
}

static const std::vector<StreamTileKernel> &stream_table()
{
    static const std::vector<StreamTileKernel> t = [] {
        std::vector<StreamTileKernel> v;
        register_tiles_stream(v);
        return v;
    }();
    return t;
}

const StreamTileKernel *find_stream(int L, int R, int C)
{
    for (const StreamTileKernel &k : stream_table())
        if (k.L == L && k.R == R && k.C == C)
            return &k;
    return nullptr;
}

static const std::vector<PersistTileKernel> &persist_table()
{
    static const std::vector<PersistTileKernel> t = [] {
        std::vector<PersistTileKernel> v;
        register_tiles_persist(v);
        return v;
    }();
    return t;
}

const PersistTileKernel *find_persist(int L, int R, int C, int lmap, int smap)
{
    for (const PersistTileKernel &k : persist_table())
        if (k.L == L && k.R == R && k.C == C && k.lmap == lmap && k.smap == smap)
            return &k;
    return nullptr;
}

const TileKernel *find_tile(int L, int lmap, int smap, int C, int R, int Q)
{
    if (C == 0 && R == 0 && Q == 0 && t_opts) {
        for (const TileKernel &k : t_opts->tiles)
            if (k.L == L && k.lmap == lmap && k.smap == smap) {
                C = k.C;
                R = k.R;
                Q = k.Q;
            }
    }
    for (const TileKernel &k : tile_table())
        if (k.L == L && k.lmap == lmap && k.smap == smap && (C == 0 || k.C == C) && (R == 0 || k.R == R) &&
            (Q == 0 || k.Q == Q))
            return &k;
    return nullptr;
}

// ================================================================ options

thread_local const PlanOptions *t_opts = nullptr;

// Built-in defaults (mufft_gb_options_init), measured on GB300:
//  - levels 0: four-step below 2^22 points, three levels from 2^22;
//  - twiddles -1: column powers wherever the column tile has the
//    shared-memory region (one sincospif per thread plus shared-memory reads,
//    no per-element global table loads on the load/store path), else sincospif;
//  - fused B/C passes off: the separate passes measured faster (they are bound
//    by instruction issue and latency, not by the HBM traffic the fusion saves);
//  - TMA-staged column tiles off: the staged 256-point tiles run at two CTAs
//    per SM and measured 2 % (double-buffered) to 47 % (single) slower than
//    per-thread loads at four CTAs per SM (the autotuner still tries them);
//  - no resident-CTA cap, no streaming row tiles (both measured slower);
//  - split-precision products on tcgen05.mma;
//  - 2D columns: two-pass four-step from 8192 points, and from 4096 for
//    wide grids (Nx >= 4096 real, >= 8192 c2c) when the L2 hints are on;
//  - persistent tile grids wherever the tile has that variant (the
//    1024-thread 4096-point column tile);
//  - multi-pass intermediates kept in L2 by cache-policy hints and dropped
//    without write-back once read (2^24 c2c 144.2 -> 135.2 us).
static int opt_field(int PlanOptions::*f, int def)
{
    return (t_opts && t_opts->*f != -2) ? t_opts->*f : def;
}
int opt_levels() { return opt_field(&PlanOptions::levels, 0); }
int opt_twiddle() { return opt_field(&PlanOptions::twiddle, -1); }
int opt_fused() { return opt_field(&PlanOptions::fused, 0); }
int opt_tma() { return opt_field(&PlanOptions::tma, 0); }
int opt_occ() { return opt_field(&PlanOptions::occ, 0); }
int opt_stream() { return opt_field(&PlanOptions::stream, 0); }
int opt_split_engine() { return opt_field(&PlanOptions::split_engine, 0); }
int opt_cols2d() { return opt_field(&PlanOptions::cols2d, 0); }
int opt_persist() { return opt_field(&PlanOptions::persist, 1); }
int opt_l2() { return opt_field(&PlanOptions::l2, 1); }

bool public_options(const mufft_gb_options *in, mufft_gb_options *o)
{
    if (!in) {
        mufft_gb_options_init(o);
        return true;
    }
    if (in->size != sizeof(mufft_gb_options)) {
        set_error(MUFFT_GB_ERR_INVALID, "options not initialised by mufft_gb_options_init");
        return false;
    }
    *o = *in;
    auto pow2_range = [](unsigned v) { return v == 0 || (is_pow2(v) && v >= 16384 && v <= 65536); };
    const char *bad = nullptr;
    if (o->multipass_levels != 0 && o->multipass_levels != 2 && o->multipass_levels != 3)
        bad = "multipass_levels must be 0 (automatic), 2 or 3";
    else if (o->twiddle_table < -1 || o->twiddle_table > 2)
        bad = "twiddle_table must be -1 (automatic), 0, 1 or 2";
    else if (o->fused_passes < 0 || o->fused_passes > 1)
        bad = "fused_passes must be 0 or 1";
    else if (o->tma < 0 || o->tma > 2)
        bad = "tma must be 0 (off), 1 (double-buffered) or 2 (single buffer)";
    else if (o->tile_occupancy < 0 || o->tile_occupancy > 32)
        bad = "tile_occupancy must be 0 (no cap) .. 32";
    else if (o->stream_tiles < 0 || o->stream_tiles > 1)
        bad = "stream_tiles must be 0 or 1";
    else if (o->split_engine < 0 || o->split_engine > 1)
        bad = "split_engine must be 0 (tcgen05) or 1 (mma.sync)";
    else if (o->columns_2d < 0 || o->columns_2d > 2)
        bad = "columns_2d must be 0 (automatic), 1 (one pass) or 2 (two passes)";
    else if (!pow2_range(o->conv_split) || !pow2_range(o->conv_classes))
        bad = "conv_split and conv_classes must be 0 or powers of two in 16384..65536";
    else if (o->stream_conv_ranges > (1u << 20))
        bad = "at most 2^20 partition ranges";
    else if (o->stream_conv_fused < 0 || o->stream_conv_fused > 1)
        bad = "stream_conv_fused must be 0 or 1";
    else if (o->fft_split != 0 && (!is_pow2(o->fft_split) || o->fft_split < 8192 || o->fft_split > 65536))
        bad = "fft_split must be 0 or a power of two in 8192..65536";
    else if (o->persistent_tiles < -1 || o->persistent_tiles > 1)
        bad = "persistent_tiles must be -1 (automatic), 0 or 1";
    else if (o->l2_residency < -1 || o->l2_residency > 1)
        bad = "l2_residency must be -1 (automatic), 0 or 1";
    else if (o->ntiles > MUFFT_GB_MAX_TILE_CHOICES)
        bad = "at most MUFFT_GB_MAX_TILE_CHOICES tile choices";
    if (bad) {
        set_error(MUFFT_GB_ERR_INVALID, "%s", bad);
        return false;
    }
    return true;
}

bool convert_options(const mufft_gb_options *in, PlanOptions *out)
{
    mufft_gb_options o;
    if (!public_options(in, &o))
        return false;
    PlanOptions p;
    p.levels = o.multipass_levels;
    p.twiddle = o.twiddle_table;
    p.fused = o.fused_passes;
    p.tma = o.tma;
    p.occ = o.tile_occupancy;
    p.stream = o.stream_tiles;
    p.split_engine = o.split_engine;
    p.cols2d = o.columns_2d;
    p.persist = o.persistent_tiles < 0 ? -2 : o.persistent_tiles;
    p.l2 = o.l2_residency < 0 ? -2 : o.l2_residency;
    for (unsigned i = 0; i < o.ntiles; i++) {
        const mufft_gb_tile_choice &c = o.tiles[i];
        const int lmap = c.load_across ? ACROSS : ALONG, smap = c.store_across ? ACROSS : ALONG;
        const TileKernel *k = nullptr;
        for (const TileKernel &t : tile_table())
            if (t.L == (int)c.L && t.lmap == lmap && t.smap == smap &&
                (c.transforms_per_tile == 0 || t.C == (int)c.transforms_per_tile) &&
                (c.elems_per_thread == 0 || t.R == (int)c.elems_per_thread) &&
                (c.cluster_ctas == 0 || t.Q == (int)c.cluster_ctas)) {
                k = &t;
                break;
            }
        if (!k) {
            set_error(MUFFT_GB_ERR_INVALID, "no tile kernel L=%u C=%u R=%u Q=%u for that map", c.L,
                      c.transforms_per_tile, c.elems_per_thread, c.cluster_ctas);
            return false;
        }
        p.tiles.push_back(*k);
    }
    *out = p;
    return true;
}

// ======================================================== device state

std::mutex g_dev_mu;
DeviceState g_dev[kMaxDevices];

bool device_prepare(int *dev_out)
{
    int dev = -1;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        set_error(MUFFT_GB_ERR_NO_DEVICE, "no CUDA device visible");
        return false;
    }
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice"))
        return false;
    if (dev < 0 || dev >= kMaxDevices) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "device index %d out of range", dev);
        return false;
    }
    std::lock_guard<std::mutex> lock(g_dev_mu);
    DeviceState &ds = g_dev[dev];
    if (!ds.ready) {
        // W^(e*k) for e in {1, 2, 4, 8}, W = exp(-2*pi*i/(r*p)), FP64 then rounded
        std::vector<float2> h(kStageTableFloat2);
        const int radices[4] = {2, 4, 8, 16}, ps[3] = {16, 256, 4096};
        for (int r : radices)
            for (int p : ps) {
                const long long n = (long long)r * p;
                for (int k = 0; k < p; k++)
                    for (int e = 0; e < 4; e++) {
                        long long m = ((long long)(1 << e) * k) % n;
                        double ph = -2.0 * M_PI * (double)m / (double)n;
                        h[stage_table_base(r, p) + 4 * k + e] = make_float2((float)std::cos(ph), (float)std::sin(ph));
                    }
            }
        if (!cuda_ok(cudaMalloc(&ds.tw, h.size() * sizeof(float2)), "cudaMalloc(twiddles)"))
            return false;
        if (!cuda_ok(cudaMemcpy(ds.tw, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice),
                     "cudaMemcpy(twiddles)"))
            return false;
        for (const TmaTileKernel &k : tma_table())
            if (!cuda_ok(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem),
                         "cudaFuncSetAttribute(tma)"))
                return false;
        for (const TileKernel &k : tile_table()) {
            if (k.smem > 48 * 1024) {
                if (!cuda_ok(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)k.smem),
                             "cudaFuncSetAttribute"))
                    return false;
                if (k.fn_c2r && !cuda_ok(cudaFuncSetAttribute(k.fn_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                              (int)k.smem),
                                         "cudaFuncSetAttribute"))
                    return false;
            }
        }
        ds.ready = true;
    }
    *dev_out = dev;
    return true;
}

std::vector<float2> r2c_twiddles(int dir, unsigned M)
{
    std::vector<float2> t(M);
    for (unsigned k = 0; k < M; k++) {
        double ph = (M_PI * dir * (double)k) / (double)M;
        double c = std::cos(ph), s = std::sin(ph);
        t[k] = make_float2((float)(-dir * s), (float)(dir * c));
    }
    return t;
}

float2 *upload(const std::vector<float2> &h)
{
    float2 *d = nullptr;
    if (!cuda_ok(cudaMalloc(&d, h.size() * sizeof(float2)), "cudaMalloc(table)"))
        return nullptr;
    if (!cuda_ok(cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice),
                 "cudaMemcpy(table)")) {
        cudaFree(d);
        return nullptr;
    }
    return d;
}

bool is_device_accessible(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

void mufft_gb_options_init(mufft_gb_options *o)
{
    if (!o)
        return;
    memset(o, 0, sizeof(*o));
    o->size = sizeof(*o);
    o->multipass_levels = 0;
    o->twiddle_table = -1;
    o->conv_split = 65536;
    o->conv_classes = 16384;
    o->stream_conv_ranges = 0;
    o->stream_conv_fused = 1;
    o->fft_split = 8192;
    o->persistent_tiles = -1;
    o->l2_residency = -1;
}

// ================================================================ memory

void *mufft_alloc(size_t size)
{
    void *p = nullptr;
    if (!cuda_ok(cudaMallocHost(&p, size ? size : 1), "cudaMallocHost"))
        return nullptr;
    return p;
}

void *mufft_calloc(size_t size)
{
    void *p = mufft_alloc(size);
    if (p)
        memset(p, 0, size);
    return p;
}

void mufft_free(void *ptr)
{
    if (!ptr)
        return;
    // mufft_alloc memory is page-locked host memory; anything else a caller
    // passes (malloc memory, as the reference's mufft_free accepts, or device
    // memory) goes back where it came from
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
        cudaGetLastError();
        free(ptr);
        return;
    }
    switch (at.type) {
    case cudaMemoryTypeHost: cudaFreeHost(ptr); break;
    case cudaMemoryTypeDevice:
    case cudaMemoryTypeManaged: cudaFree(ptr); break;
    default: free(ptr); break;
    }
}

void *mufft_gb_device_alloc(size_t size)
{
    void *p = nullptr;
    if (!cuda_ok(cudaMalloc(&p, size ? size : 1), "cudaMalloc"))
        return nullptr;
    return p;
}

void mufft_gb_device_free(void *ptr)
{
    if (ptr)
        cudaFree(ptr);
}

int mufft_gb_memcpy(void *dst, const void *src, size_t size)
{
    if (!cuda_ok(cudaMemcpy(dst, src, size, cudaMemcpyDefault), "cudaMemcpy"))
        return t_err;
    return MUFFT_GB_OK;
}

int mufft_gb_device_synchronize(void)
{
    if (!cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize"))
        return t_err;
    return MUFFT_GB_OK;
}

int mufft_gb_list_tiles(char *buf, size_t size)
{
    std::string s;
    char line[160];
    for (const TileKernel &k : tile_table()) {
        snprintf(line, sizeof(line), "%sL=%d R=%d C=%d Q=%d %s/%s threads=%d smem=%zu", s.empty() ? "" : "; ", k.L,
                 k.R, k.C, k.Q, k.lmap ? "across" : "along", k.smap ? "across" : "along", k.threads, k.smem);
        s += line;
    }
    if (buf && size)
        snprintf(buf, size, "%s", s.c_str());
    return (int)s.size();
}

// ================================================================ errors

int mufft_gb_last_error(void) { return t_err; }
const char *mufft_gb_last_error_string(void) { return t_err ? t_errmsg : ""; }
void mufft_gb_clear_error(void)
{
    t_err = 0;
    t_errmsg[0] = 0;
}

}  // extern "C"
