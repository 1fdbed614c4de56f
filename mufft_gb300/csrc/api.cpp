// Host side of libmufft_gb300: the muFFT C API (fft.h) and its GB300
// extensions (mufft_gb300.h).
//
// Plan creation mirrors the reference constructors (fft.c:441-792): the same
// argument checks and NULL returns, the same buffer-size contracts.  Where the
// reference builds a list of CPU passes (fft.c:325-435), this file builds a
// list of GPU launches:
//   - complex length M <= 16384: one tile-FFT launch (one HBM read + write per
//     transform), with the r2c/c2r fix-up and the convolution multiply fused
//     into its load or store phase;
//   - M > 16384: a four-step pair, M = N1 x N2: column FFTs of length N1 with
//     the W_M^(k1*n2) twiddle fused into their stores, then row FFTs of length
//     N2 with transposed stores into natural order.
// Executes enqueue those launches on a stream.  The fft.h executes stage host
// buffers through plan-owned device memory and synchronise before returning,
// like the reference's synchronous calls (fft.c:811-989).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/fft.h"
#include "../../include/mufft_gb300.h"
#include "bc_fused.h"
#include "common.h"
#include "conv_ragged.h"
#include "misc_kernels.h"
#include "split_tc.h"
#include "tiles_tma.h"
#include "tiles_stream.h"
#include "stream_conv.h"
#include "registry.h"

using namespace mgb;

// ================================================================ errors

namespace {

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

bool is_pow2(unsigned n) { return n != 0 && (n & (n - 1)) == 0; }

unsigned ilog2u(unsigned long long n)
{
    unsigned l = 0;
    while ((1ull << l) < n)
        l++;
    return l;
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        if (dev >= 0 && dev != prev)
            cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
            cudaSetDevice(prev);
    }
};

}  // namespace

// ============================================================= registry

namespace mgb {

static std::vector<TileKernel> &tile_table()
{
    static std::vector<TileKernel> t = [] {
        std::vector<TileKernel> v;
        register_tiles_along(v);
        register_tiles_across(v);
        register_tiles_transpose(v);
        return v;
    }();
    return t;
}

static std::vector<TmaTileKernel> &tma_table()
{
    static std::vector<TmaTileKernel> t = [] {
        std::vector<TmaTileKernel> v;
        register_tiles_tma(v);
        return v;
    }();
    return t;
}

static const TmaTileKernel *find_tma(int L, int R, int C, int nbuf)
{
    for (const TmaTileKernel &k : tma_table())
        if (k.L == L && k.R == R && k.C == C && k.nbuf == nbuf)
            return &k;
    return nullptr;
}

static std::vector<StreamTileKernel> &stream_table()
{
    static std::vector<StreamTileKernel> t = [] {
        std::vector<StreamTileKernel> v;
        register_tiles_stream(v);
        return v;
    }();
    return t;
}

static const StreamTileKernel *find_stream(int L, int R, int C)
{
    for (const StreamTileKernel &k : stream_table())
        if (k.L == L && k.R == R && k.C == C)
            return &k;
    return nullptr;
}

static std::mutex g_choice_mu;
static std::vector<TileKernel> g_choice;  // preferred (L, lmap, smap) -> C

// Schedule choices of one plan (the autotuner's unit): -2 leaves a knob at its
// process-wide setting; `tiles` are preferred (L, lmap, smap) -> (C, R, Q).
struct PlanOptions {
    int levels = -2, twiddle = -2, fused = -2, tma = -2, occ = -2, stream = -2;
    std::vector<TileKernel> tiles;
};
// Set while a plan is built with explicit choices (candidate or remembered).
thread_local const PlanOptions *t_opts = nullptr;

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
    if (C == 0 && R == 0 && Q == 0) {
        std::lock_guard<std::mutex> lock(g_choice_mu);
        for (const TileKernel &k : g_choice)
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

bool set_tile_choice(int L, int lmap, int smap, int C, int R, int Q)
{
    if ((C != 0 || R != 0 || Q != 0) && !find_tile(L, lmap, smap, C, R, Q))
        return false;
    std::lock_guard<std::mutex> lock(g_choice_mu);
    for (auto it = g_choice.begin(); it != g_choice.end(); ++it)
        if (it->L == L && it->lmap == lmap && it->smap == smap) {
            g_choice.erase(it);
            break;
        }
    if (C != 0 || R != 0 || Q != 0) {
        TileKernel k{};
        k.L = L;
        k.lmap = lmap;
        k.smap = smap;
        k.C = C;
        k.R = R;
        k.Q = Q;
        g_choice.push_back(k);
    }
    return true;
}

}  // namespace mgb

// ======================================================== device state

namespace {

constexpr int kMaxDevices = 64;

struct DeviceState {
    bool ready = false;
    float2 *tw = nullptr;  // stage twiddle table (common.h: stage_table_base)
};

std::mutex g_dev_mu;
DeviceState g_dev[kMaxDevices];

// Makes sure the current device has its twiddle table and kernel attributes.
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

// Host-generated FP64 tables, rounded once to float.
std::vector<float2> r2c_twiddles(int dir, unsigned M)
{
    // i*dir*exp(i*pi*dir*k/M) (fft.c:441-455)
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

// ================================================================ passes

enum Role { ROLE_NONE = 0, ROLE_IN, ROLE_OUT, ROLE_IN2, ROLE_SCRATCH, ROLE_SCRATCH2 };
enum PassType { PASS_TILE = 0, PASS_R2C_FIXUP = 1, PASS_BC = 2, PASS_SPLIT = 3 };

struct Pass {
    PassType type = PASS_TILE;
    const TileKernel *k = nullptr;
    TileArgs a{};
    Role in_role = ROLE_IN, out_role = ROLE_OUT, in2_role = ROLE_NONE;
    dim3 grid;
    // in-place r2c fix-up
    long long M = 0, dist = 0;
    unsigned batch = 1;
    int full = 0;
    // fused B/C passes (bc_fused.cu): y is the scratch, x the role out_role
    BcArgs bc{};
    size_t bc_counter_bytes = 0;
    unsigned bc_grid = 0;
    // column tile with TMA-staged input (tiles_tma.cu), used when the input
    // layout allows it at launch; `k` is the fallback
    const TmaTileKernel *tk = nullptr;
    unsigned tma_grid = 0;
    int *tma_err = nullptr;
    // split-precision tensor-core transform (split_tc.cu, split_umma.cu)
    SplitArgs sp{};
    int sp_stages = 0, sp_limbs = 0, sp_engine = 0;
    unsigned sp_grid = 0;
    // resident-CTA cap: tile launches request at least this much dynamic
    // shared memory (0: the kernel's own need)
    size_t smem_min = 0;
    // row tiles as persistent CTAs streaming their tiles (tiles_stream.cu);
    // `k` is the same tile as one launch per tile
    const StreamTileKernel *sk = nullptr;
    unsigned sk_grid = 0;
};

struct Buffers {
    const void *in;
    void *out;
    const void *in2;
    void *scratch;
    void *scratch2 = nullptr;
};

const void *pick(Role r, const Buffers &b)
{
    switch (r) {
    case ROLE_IN: return b.in;
    case ROLE_OUT: return b.out;
    case ROLE_IN2: return b.in2;
    case ROLE_SCRATCH: return b.scratch;
    case ROLE_SCRATCH2: return b.scratch2;
    default: return nullptr;
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeTiledFn) nullptr;
        }
        return (EncodeTiledFn)f;
    }();
    return fn;
}

// Tensor map of a column pass's input: {columns, L rows, row blocks} of
// 8-byte elements, box {C, L, 1}.  False when the layout does not fit TMA's
// rules (16-byte aligned base and strides, unit column distance, plain
// prologue, uniform block stride); the pass then runs its regular kernel.
bool tma_map_for(const Pass &p, const float2 *in, CUtensorMap *map)
{
    const TileArgs &a = p.a;
    if (a.prologue != PRO_PLAIN || a.in_dist != 1 || ((uintptr_t)in & 15) || (a.in_stride & 1) || a.in_stride <= 0)
        return false;
    long long bstride = a.in_batch;
    if (a.ysplit && a.in_batch2 != (long long)a.ysplit * a.in_batch)
        return false;
    if (p.grid.y <= 1)
        bstride = a.in_stride * p.tk->L;
    if (bstride & 1 || bstride < a.in_stride * p.tk->L)
        return false;
    EncodeTiledFn enc = encode_tiled();
    if (!enc)
        return false;
    const cuuint64_t dims[3] = {a.ntrans, (cuuint64_t)p.tk->L, p.grid.y > 0 ? p.grid.y : 1};
    const cuuint64_t strides[2] = {(cuuint64_t)a.in_stride * 8, (cuuint64_t)bstride * 8};
    const cuuint32_t box[3] = {(cuuint32_t)p.tk->C, (cuuint32_t)p.tk->L, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, (void *)in, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t run_passes(const std::vector<Pass> &ps, const Buffers &b, cudaStream_t st, size_t first = 0,
                       size_t count = (size_t)-1)
{
    for (size_t i = first; i < ps.size() && i - first < count; i++) {
        const Pass &p = ps[i];
        if (p.type == PASS_TILE) {
            if ((p.k->lmap == ALONG && p.a.in_stride != 1) || (p.k->smap == ALONG && p.a.out_stride != 1))
                return cudaErrorInvalidValue;  // ALONG phases assume unit stride
            TileArgs a = p.a;
            a.in = (const float2 *)pick(p.in_role, b);
            a.out = (float2 *)pick(p.out_role, b);
            a.in2 = (const float2 *)pick(p.in2_role, b);
            if (p.tk) {
                CUtensorMap map;
                if (tma_map_for(p, a.in, &map)) {
                    const unsigned tiles_x = (a.ntrans + p.tk->C - 1) / p.tk->C;
                    unsigned ntiles = tiles_x * p.grid.y;
                    int *err = p.tma_err;
                    void *targs[] = {&map, &a, (void *)&tiles_x, &ntiles, &err};
                    const unsigned grid = std::min(ntiles, p.tma_grid);
                    cudaError_t e = cudaLaunchKernel(p.tk->fn, dim3(grid), dim3(p.tk->threads), targs, p.tk->smem, st);
                    if (e != cudaSuccess)
                        return e;
                    continue;
                }
            }
            if (p.sk) {
                unsigned ntiles = p.grid.x;
                void *sargs[] = {&a, &ntiles};
                cudaError_t e = cudaLaunchKernel(p.sk->fn, dim3(p.sk_grid), dim3(p.sk->threads), sargs, p.sk->smem, st);
                if (e != cudaSuccess)
                    return e;
                continue;
            }
            void *args[] = {&a};
            const size_t smem =
                std::max((a.tw_lo || a.tw_colpow || a.tw_by_y) ? p.k->smem : p.k->smem_ex, p.smem_min);
            cudaError_t e;
            if (p.k->Q > 1) {
                // one tile per cluster of Q CTAs (distributed shared memory)
                cudaLaunchConfig_t cfg = {};
                cudaLaunchAttribute attr[1];
                cfg.gridDim = dim3(p.grid.x * p.k->Q, p.grid.y, p.grid.z);
                cfg.blockDim = dim3(p.k->threads);
                cfg.dynamicSmemBytes = smem;
                cfg.stream = st;
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = p.k->Q;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                e = cudaLaunchKernelExC(&cfg, p.k->fn, args);
            } else {
                // c2r fix-up rows staged in shared memory where the tile has that variant
                const bool c2r_rows = p.k->fn_c2r && (a.prologue == PRO_C2R || a.prologue == PRO_MUL_C2R) &&
                                      a.mirror_ldist == 0 && a.mirror_len == p.k->L && !a.half && a.in_stride == 1;
                e = cudaLaunchKernel(c2r_rows ? p.k->fn_c2r : p.k->fn, p.grid, dim3(p.k->threads), args, smem, st);
            }
            if (e != cudaSuccess)
                return e;
        } else if (p.type == PASS_SPLIT) {
            SplitArgs a = p.sp;
            a.in = (const float2 *)pick(p.in_role, b);
            a.out = (float2 *)pick(p.out_role, b);
            // bulk async copies need 16-byte aligned transforms
            a.bulk = (((uintptr_t)a.in & 15) == 0 && (a.in_dist & 1) == 0) ? 1 : 0;
            void *args[] = {&a};
            cudaError_t e =
                p.sp_engine == 0
                    ? cudaLaunchKernel(split_umma_kernel(p.sp_stages, p.sp_limbs), dim3(p.sp_grid),
                                       dim3(split_umma_threads()), args, split_umma_smem_bytes(), st)
                    : cudaLaunchKernel(split_kernel(p.sp_stages, p.sp_limbs), dim3(p.sp_grid), dim3(kSplitThreads),
                                       args, split_smem_bytes(), st);
            if (e != cudaSuccess)
                return e;
        } else if (p.type == PASS_BC) {
            BcArgs a = p.bc;
            a.y = (const float2 *)b.scratch;
            a.x = (float2 *)pick(p.out_role, b);
            cudaError_t e = cudaMemsetAsync(a.counters, 0, p.bc_counter_bytes, st);
            if (e != cudaSuccess)
                return e;
            void *args[] = {&a};
            e = cudaLaunchKernel(bc_kernel(), dim3(p.bc_grid), dim3(bc_threads()), args, bc_smem_bytes(), st);
            if (e != cudaSuccess)
                return e;
        } else {
            cudaError_t e = launch_r2c_fixup_inplace((float2 *)pick(p.out_role, b), p.a.rtw, p.M, p.dist,
                                                     p.batch, p.full, st);
            if (e != cudaSuccess)
                return e;
        }
    }
    return cudaSuccess;
}

const char *pro_name(int p)
{
    static const char *n[] = {"plain", "c2r", "mul", "mul_c2r"};
    return (p >= 0 && p < 4) ? n[p] : "?";
}
const char *epi_name(int e)
{
    static const char *n[] = {"plain", "r2c", "r2c_full", "twiddle"};
    return (e >= 0 && e < 4) ? n[e] : "?";
}

std::string describe(const std::vector<Pass> &ps)
{
    std::string s;
    char buf[256];
    for (size_t i = 0; i < ps.size(); i++) {
        const Pass &p = ps[i];
        if (p.type == PASS_TILE)
            snprintf(buf, sizeof(buf), "%stile%s L=%d R=%d C=%d Q=%d %s/%s grid=%ux%u threads=%d smem=%zu pro=%s%s epi=%s%s conj=%d",
                     i ? "; " : "", p.tk ? (p.tk->nbuf == 2 ? "+tma2" : "+tma1") : (p.sk ? "+stream" : ""), p.k->L, p.k->R, p.k->C, p.k->Q, p.k->lmap ? "across" : "along",
                     p.k->smap ? "across" : "along", p.sk ? p.sk_grid : p.grid.x, p.grid.y, p.k->threads, std::max(p.k->smem, p.smem_min),
                     pro_name(p.a.prologue), p.a.half ? "+half" : "", epi_name(p.a.epilogue),
                     p.a.epilogue != EPI_TWIDDLE ? "" : (p.a.tw_colpow ? "/colpow" : (p.a.tw_lo ? "/table" : "/sincos")),
                     p.a.conj);
        else if (p.type == PASS_SPLIT)
            snprintf(buf, sizeof(buf), "%ssplit_tc N=%d bf16x%d %s grid=%u threads=%d smem=%zu conj=%d", i ? "; " : "",
                     1 << (4 * p.sp_stages), p.sp_limbs, p.sp_engine == 0 ? "tcgen05" : "mma.sync", p.sp_grid,
                     p.sp_engine == 0 ? split_umma_threads() : kSplitThreads,
                     p.sp_engine == 0 ? split_umma_smem_bytes() : split_smem_bytes(), p.sp.conj);
        else if (p.type == PASS_BC)
            snprintf(buf, sizeof(buf), "%sfused_bc 256x256 rows=%u blocks=%u ring=%u grid=%u", i ? "; " : "",
                     p.bc.n1, p.bc.nblk, p.bc.ring_slots, p.bc_grid);
        else
            snprintf(buf, sizeof(buf), "%sr2c_fixup M=%lld batch=%u full=%d", i ? "; " : "", p.M, p.batch, p.full);
        s += buf;
    }
    return s;
}

// One complex FFT stage group: `batch` transforms of length M.
struct FftSpec {
    unsigned M = 0;
    unsigned batch = 1;
    long long in_dist = 0, out_dist = 0;  // float2 units
    int prologue = PRO_PLAIN;
    int half = 0;
    int epilogue = EPI_PLAIN;             // PLAIN, R2C or R2C_FULL
    int conj_in = 0, conj_out = 0;
    Role in_role = ROLE_IN, out_role = ROLE_OUT, in2_role = ROLE_NONE;
    float scale = 1.0f;
    int conj2 = 0;                        // multiply by conj(in2): adjoint convolution
};

// Device tables and scratch a schedule needs; allocated unless `dry`.
struct PlanResources {
    float2 *rtw = nullptr;
    float2 *twlo = nullptr;   // multi-pass: W_M^(k*c) of the first column pass
    float2 *twlo2 = nullptr;  // three-level: the same for the second column pass
    float2 *scratch = nullptr;
    size_t scratch_bytes = 0;
    float2 *scratch2 = nullptr;   // 2D plans whose columns run as a two-pass four-step
    float2 *ring = nullptr;       // fused B/C: L2-resident ring of row blocks
    unsigned *counters = nullptr; // fused B/C: task counters
    int *err = nullptr;           // device error flag of bounded waits
    unsigned *afrag = nullptr;    // split precision: DFT-16 limbs in mma fragment order
    float2 *sptw = nullptr;       // split precision: stage twiddles
    void *bfrag = nullptr;        // split precision (tcgen05): DFT-16 limbs as B operands
    void release()
    {
        cudaFree(afrag);
        cudaFree(sptw);
        cudaFree(bfrag);
        afrag = nullptr;
        sptw = nullptr;
        bfrag = nullptr;
        cudaFree(rtw);
        cudaFree(twlo);
        cudaFree(twlo2);
        cudaFree(scratch);
        cudaFree(scratch2);
        cudaFree(ring);
        cudaFree(counters);
        cudaFree(err);
        rtw = twlo = twlo2 = scratch = scratch2 = ring = nullptr;
        counters = nullptr;
        err = nullptr;
    }
};

// Multi-pass depth for transforms longer than one tile: 0 = automatic
// (set with mufft_gb_set_multipass_levels).
std::atomic<int> g_levels{0};
// Four-step twiddles of column passes: sincospif per element (0), the
// per-plan table times a per-tile factor (1), or per-tile column powers (2).
// Automatic (-1): column powers wherever the tile has the shared-memory
// region -- one sincospif per thread plus shared-memory reads, no per-element
// global table loads on the load/store path.
std::atomic<int> g_twiddle_table{-1};
// Fuse the last two passes of M = N1 x 65536 transforms into one persistent
// launch with an L2-resident intermediate (1), or run them separately (0,
// default: the separate passes measured faster on GB300 -- they are bound by
// instruction issue and latency, not by the HBM traffic the fusion saves).
std::atomic<int> g_fused_bc{0};
// 2D columns: 0 automatic (two-pass four-step from 8192 points), 1 one column
// pass, 2 the two-pass form whenever possible (set with mufft_gb_set_2d_columns).
std::atomic<int> g_2d_columns{0};
// Split-precision products on tcgen05.mma (0, default) or warp-level mma.sync (1).
std::atomic<int> g_split_engine{0};

// Column passes with TMA-staged inputs: 1 double-buffered, 2 single buffer,
// 0 off (default: on GB300 the staged 256-point column tiles run at two CTAs
// per SM and measured 2 % (double-buffered) to 47 % (single) slower than the
// per-thread loads at four CTAs per SM; the autotuner still tries them).
std::atomic<int> g_tma{0};
int opt_tma() { return (t_opts && t_opts->tma != -2) ? t_opts->tma : g_tma.load(); }
int opt_twiddle() { return (t_opts && t_opts->twiddle != -2) ? t_opts->twiddle : g_twiddle_table.load(); }
int opt_levels() { return (t_opts && t_opts->levels != -2) ? t_opts->levels : g_levels.load(); }
int opt_fused() { return (t_opts && t_opts->fused != -2) ? t_opts->fused : g_fused_bc.load(); }
// Resident tile CTAs per SM (0: as many as fit).  A cap spreads a grid that
// would fill the GPU about once over several waves, so that CTAs loading
// their inputs overlap CTAs storing their outputs.
std::atomic<int> g_occ{0};
int opt_occ() { return (t_opts && t_opts->occ != -2) ? t_opts->occ : g_occ.load(); }
// Row tiles of one launch per tile (0) or persistent streaming CTAs (1).
std::atomic<int> g_stream{0};
int opt_stream() { return (t_opts && t_opts->stream != -2) ? t_opts->stream : g_stream.load(); }

bool use_twiddle_table(const TileKernel *k)
{
    const int t = opt_twiddle();
    return k->has_thi && t == 1;
}

// Column powers (mode 2, and the automatic choice wherever the tile has the
// shared-memory region): the twiddles of a column are W^(col*base) of each
// thread times R per-column powers computed once per tile.
bool use_colpow(const TileKernel *k)
{
    const int t = opt_twiddle();
    return k->has_thi && (t == 2 || t < 0);
}

// W_M^(k*c) for k < L, c < C: the per-column half of a four-step twiddle.
bool upload_twlo(unsigned L, int C, unsigned long long M, float2 *&dst)
{
    std::vector<float2> lo((size_t)L * C);
    for (unsigned k = 0; k < L; k++)
        for (int c = 0; c < C; c++) {
            double ph = -2.0 * M_PI * (double)((unsigned long long)k * c % M) / (double)M;
            lo[(size_t)k * C + c] = make_float2((float)std::cos(ph), (float)std::sin(ph));
        }
    dst = upload(lo);
    return dst != nullptr;
}

// Column pass of a multi-pass transform: `ncols` columns of length L (stride
// `stride`), output twiddled by W_Mtw^(k*column).
Pass column_pass(const TileKernel *k, const float2 *tw, unsigned L, unsigned ncols, long long stride,
                 unsigned long long Mtw, const float2 *twlo)
{
    Pass p;
    p.k = k;
    p.a.in_stride = p.a.out_stride = stride;
    p.a.in_dist = p.a.out_dist = 1;
    p.a.ntrans = ncols;
    p.a.epilogue = EPI_TWIDDLE;
    p.a.tw = tw;
    p.a.tw_scale = 2.0f / (float)Mtw;
    p.a.tw_mask = (unsigned)(Mtw - 1);
    p.a.tw_lo = use_twiddle_table(k) ? twlo : nullptr;
    p.a.tw_colpow = use_colpow(k) ? 1 : 0;
    p.a.scale = 1.0f;
    (void)L;
    return p;
}

// Gives every column pass whose tile has a TMA-staged variant that variant
// (persistent grid: SMs x resident CTAs); the regular kernel stays as the
// fallback for layouts TMA cannot describe.
bool attach_tma(std::vector<Pass> &ps, PlanResources &res, bool dry, int device)
{
    const int mode = opt_tma();
    if (mode == 0)
        return true;
    for (Pass &p : ps) {
        if (p.type != PASS_TILE || !p.k || p.k->Q != 1 || p.k->lmap != ACROSS || p.k->smap != ACROSS)
            continue;
        const TmaTileKernel *tk = find_tma(p.k->L, p.k->R, p.k->C, mode == 2 ? 1 : 2);
        if (!tk)
            continue;
        p.tk = tk;
        if (dry) {
            p.tma_grid = 2 * 152;
            continue;
        }
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tk->fn, tk->threads, tk->smem),
                     "occupancy(tma)"))
            return false;
        p.tma_grid = (unsigned)(sms * std::max(per_sm, 1));
        if (!res.err && (!cuda_ok(cudaMalloc(&res.err, sizeof(int)), "cudaMalloc(err)") ||
                         !cuda_ok(cudaMemset(res.err, 0, sizeof(int)), "cudaMemset(err)")))
            return false;
        p.tma_err = res.err;
    }
    return true;
}

// Gives every contiguous row-tile pass (one batch dimension, unit strides)
// that has a streaming variant that variant: a persistent grid of SMs x
// resident CTAs whose CTAs prefetch their next tile's inputs.
bool attach_stream(std::vector<Pass> &ps, bool dry, int device)
{
    if (opt_stream() != 1)
        return true;
    for (Pass &p : ps) {
        if (p.type != PASS_TILE || !p.k || p.k->Q != 1 || p.k->lmap != ALONG || p.k->smap != ALONG || p.tk ||
            p.grid.y != 1 || p.a.ysplit || p.a.in_stride != 1 || p.a.out_stride != 1)
            continue;
        const StreamTileKernel *sk = find_stream(p.k->L, p.k->R, p.k->C);
        if (!sk)
            continue;
        int sms = 152, per_sm = 1;
        if (!dry) {
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            if (sk->smem > 48 * 1024 &&
                !cuda_ok(cudaFuncSetAttribute(sk->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sk->smem),
                         "cudaFuncSetAttribute(stream)"))
                return false;
            if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sk->fn, sk->threads, sk->smem),
                         "occupancy(stream)"))
                return false;
        }
        p.sk = sk;
        p.sk_grid = std::min(p.grid.x, (unsigned)(sms * std::max(per_sm, 1)));
    }
    return true;
}

// Applies the resident-CTA cap to every single-CTA tile pass: the launch
// asks for enough dynamic shared memory that at most `occ` CTAs fit per SM.
bool attach_occupancy(std::vector<Pass> &ps, bool dry, int device)
{
    const int occ = opt_occ();
    if (occ <= 0)
        return true;
    int per_sm = 233472, optin = 232448;
    if (!dry) {
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    }
    // each resident CTA also takes 1 KiB of reserved shared memory
    const int w = std::min(per_sm / occ - 1024, optin);
    if (w <= 0)
        return true;
    const size_t want = (size_t)w & ~(size_t)127;
    for (Pass &p : ps) {
        if (p.type != PASS_TILE || !p.k || p.k->Q != 1 || p.tk || p.sk)
            continue;
        if (want <= p.k->smem)
            continue;
        p.smem_min = want;
        if (!dry && (!cuda_ok(cudaFuncSetAttribute(p.k->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin),
                              "cudaFuncSetAttribute(occupancy)") ||
                     (p.k->fn_c2r && !cuda_ok(cudaFuncSetAttribute(p.k->fn_c2r,
                                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, optin),
                                              "cudaFuncSetAttribute(occupancy)"))))
            return false;
    }
    return true;
}

bool build_fft_passes(const FftSpec &s, const float2 *tw, PlanResources &res, bool dry,
                      std::vector<Pass> &out)
{
    const unsigned M = s.M;
    const bool r2c = s.epilogue == EPI_R2C || s.epilogue == EPI_R2C_FULL;
    if (M <= kMaxSinglePass) {
        const TileKernel *k = find_tile((int)M, ALONG, ALONG);
        if (!k) {
            set_error(MUFFT_GB_ERR_UNSUPPORTED, "no tile kernel for length %u", M);
            return false;
        }
        Pass p;
        p.k = k;
        p.a.in_stride = 1;
        p.a.in_dist = s.in_dist;
        p.a.out_stride = 1;
        p.a.out_dist = s.out_dist;
        p.a.ntrans = s.batch;
        p.a.conj = (s.conj_in ? 1 : 0) | (s.conj_out ? 2 : 0);
        p.a.prologue = s.prologue;
        p.a.half = s.half;
        p.a.epilogue = s.epilogue;
        p.a.tw = tw;
        p.a.rtw = res.rtw;
        p.a.mirror_len = M;
        p.a.mirror_ldist = 0;
        p.a.scale = s.scale;
        p.in_role = s.in_role;
        p.out_role = s.out_role;
        p.in2_role = s.in2_role;
        p.a.conj2 = s.conj2;
        p.grid = dim3((s.batch + k->C - 1) / k->C, 1);
        out.push_back(p);
        return true;
    }

    const unsigned lg = ilog2u(M);
    int levels = opt_levels();
    if (levels == 0)
        levels = lg >= 22 ? 3 : 2;  // measured crossover on GB300
    if (levels == 3 && lg >= 20 && opt_fused()) {
        // M = N1 x 65536: pass A column tiles of length N1, then the fused
        // persistent B/C launch with an L2-resident intermediate.
        const unsigned N1 = M >> 16;
        const TileKernel *ka = find_tile((int)N1, ACROSS, ACROSS);
        if (ka && N1 % 16 == 0 && s.batch <= 65535) {
            const unsigned long long MR = 65536;
            const unsigned blk_per_item = N1 / 16;
            const unsigned nblk = blk_per_item * s.batch;
            const unsigned ring = nblk < 2 ? 1 : (nblk < 4 ? 2 : 4);
            Pass pbc;
            pbc.type = PASS_BC;
            pbc.out_role = s.out_role;
            pbc.bc.n1 = N1;
            pbc.bc.nblk = nblk;
            pbc.bc.blk_per_item = blk_per_item;
            pbc.bc.ring_slots = ring;
            pbc.bc.y_item = M;
            pbc.bc.x_item = s.out_dist;
            pbc.bc_counter_bytes = (2 * (size_t)nblk + 1) * sizeof(unsigned);
            const TileKernel *kb = find_tile(256, ACROSS, ACROSS, 16, 16, 1);
            float2 *twlo_b = nullptr;
            if (!dry) {
                res.scratch_bytes = (size_t)M * s.batch * sizeof(float2);
                if (!cuda_ok(cudaMalloc(&res.scratch, res.scratch_bytes), "cudaMalloc(scratch)") ||
                    !cuda_ok(cudaMalloc(&res.ring, (size_t)ring * 16 * MR * sizeof(float2)), "cudaMalloc(ring)") ||
                    !cuda_ok(cudaMalloc(&res.counters, pbc.bc_counter_bytes), "cudaMalloc(counters)") ||
                    !cuda_ok(cudaMalloc(&res.err, sizeof(int)), "cudaMalloc(err)") ||
                    !cuda_ok(cudaMemset(res.err, 0, sizeof(int)), "cudaMemset(err)"))
                    return false;
                if ((use_twiddle_table(ka) && !upload_twlo(N1, ka->C, M, res.twlo)) ||
                    !upload_twlo(256, 16, MR, res.twlo2))
                    return false;
                twlo_b = res.twlo2;
                int dev = 0, sms = 0, per_sm = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bc_kernel(), bc_threads(),
                                                                           bc_smem_bytes()),
                             "occupancy"))
                    return false;
                pbc.bc_grid = (unsigned)(sms * (per_sm > 0 ? per_sm : 1));
            } else {
                pbc.bc_grid = 0;
            }
            pbc.bc.ring = res.ring;
            pbc.bc.counters = res.counters;
            pbc.bc.err = res.err;
            // pass-B template: 256-point columns over stride 256 in one row, W_65536 twiddle
            TileArgs &tb = pbc.bc.b;
            tb.in_stride = tb.out_stride = 256;
            tb.in_dist = tb.out_dist = 1;
            tb.ntrans = 256;
            tb.epilogue = EPI_TWIDDLE;
            tb.tw = tw;
            tb.tw_scale = 2.0f / 65536.0f;
            tb.tw_mask = 65535u;
            tb.tw_lo = (kb && kb->has_thi) ? twlo_b : nullptr;
            tb.scale = 1.0f;
            // pass-C template: 16 rows of 256 contiguous points, stores across rows
            TileArgs &tc = pbc.bc.c;
            tc.in_stride = 1;
            tc.in_dist = (long long)MR;
            tc.out_stride = (long long)N1 * 256;
            tc.out_dist = 1;
            tc.ntrans = 16;
            tc.conj = s.conj_out ? 2 : 0;
            tc.tw = tw;
            tc.scale = 1.0f;

            Pass pa = column_pass(ka, tw, N1, (unsigned)MR, (long long)MR, M, res.twlo);
            pa.a.in_batch = s.in_dist;
            pa.a.out_batch = M;
            pa.a.conj = s.conj_in ? 1 : 0;
            pa.a.prologue = s.prologue;
            pa.a.half = s.half;
            pa.a.rtw = res.rtw;
            pa.a.mirror_len = M;
            pa.a.mirror_ldist = 1;
            pa.a.scale = s.scale;
            pa.in_role = s.in_role;
            pa.in2_role = s.in2_role;
            pa.a.conj2 = s.conj2;
            pa.out_role = ROLE_SCRATCH;
            pa.grid = dim3((unsigned)((MR + ka->C - 1) / ka->C), s.batch);
            out.push_back(pa);
            out.push_back(pbc);
            if (r2c) {
                Pass p3;
                p3.type = PASS_R2C_FIXUP;
                p3.a.rtw = res.rtw;
                p3.out_role = s.out_role;
                p3.M = M;
                p3.dist = s.out_dist;
                p3.batch = s.batch;
                p3.full = s.epilogue == EPI_R2C_FULL;
                out.push_back(p3);
            }
            return true;
        }
    }
    if (levels == 3 && lg >= 12) {
        // Three levels, M = N1 * N2 * N3 (near-equal powers of two, each tile
        // small enough for several CTAs per SM):
        //   A: columns of length N1 over m < N2*N3 (stride N2*N3), twiddle W_M^(k1*m)
        //   B: in place, per row k1: columns of length N2 over n3 < N3, twiddle
        //      W_(N2*N3)^(k2*n3)
        //   C: rows (k1, k2) of length N3, stores transposed to X[k1 + N1*(k2 + N2*k3)]
        const unsigned l1 = lg / 3, l2 = (lg - l1) / 2, l3 = lg - l1 - l2;
        const unsigned N1 = 1u << l1, N2 = 1u << l2, N3 = 1u << l3;
        const unsigned long long MR = (unsigned long long)N2 * N3;
        if (s.batch > 65535u / N2 || s.batch > 65535) {
            set_error(MUFFT_GB_ERR_UNSUPPORTED, "batch %u too large for three-level lengths", s.batch);
            return false;
        }
        const TileKernel *ka = find_tile((int)N1, ACROSS, ACROSS);
        const TileKernel *kb = find_tile((int)N2, ACROSS, ACROSS);
        const TileKernel *kr = find_tile((int)N3, ALONG, ACROSS);
        if (!ka || !kb || !kr) {
            set_error(MUFFT_GB_ERR_UNSUPPORTED, "no three-level kernels for %u x %u x %u", N1, N2, N3);
            return false;
        }
        float2 *twlo_b = nullptr;
        if (!dry) {
            res.scratch_bytes = (size_t)M * s.batch * sizeof(float2);
            if (!cuda_ok(cudaMalloc(&res.scratch, res.scratch_bytes), "cudaMalloc(scratch)"))
                return false;
            if ((use_twiddle_table(ka) && !upload_twlo(N1, ka->C, M, res.twlo)) ||
                (use_twiddle_table(kb) && !upload_twlo(N2, kb->C, MR, res.twlo2)))
                return false;
            twlo_b = res.twlo2;
        }
        Pass pa = column_pass(ka, tw, N1, (unsigned)MR, (long long)MR, M, res.twlo);
        pa.a.in_batch = s.in_dist;
        pa.a.out_batch = M;
        pa.a.conj = s.conj_in ? 1 : 0;
        pa.a.prologue = s.prologue;
        pa.a.half = s.half;
        pa.a.rtw = res.rtw;
        pa.a.mirror_len = M;
        pa.a.mirror_ldist = 1;
        pa.a.scale = s.scale;
        pa.in_role = s.in_role;
        pa.in2_role = s.in2_role;
        pa.a.conj2 = s.conj2;
        pa.out_role = ROLE_SCRATCH;
        pa.grid = dim3((unsigned)((MR + ka->C - 1) / ka->C), s.batch);
        out.push_back(pa);

        Pass pb = column_pass(kb, tw, N2, N3, (long long)N3, MR, twlo_b);
        pb.a.ysplit = N1;
        pb.a.in_batch = pb.a.out_batch = (long long)MR;
        pb.a.in_batch2 = pb.a.out_batch2 = M;
        pb.in_role = ROLE_SCRATCH;
        pb.out_role = ROLE_SCRATCH;
        pb.grid = dim3((N3 + kb->C - 1) / kb->C, N1 * s.batch);
        out.push_back(pb);

        Pass pc;
        pc.k = kr;
        pc.a.in_stride = 1;
        pc.a.in_dist = (long long)MR;
        pc.a.out_stride = (long long)N1 * N2;
        pc.a.out_dist = 1;
        pc.a.ysplit = N2;
        pc.a.in_batch = N3;
        pc.a.out_batch = N1;
        pc.a.in_batch2 = M;
        pc.a.out_batch2 = s.out_dist;
        pc.a.ntrans = N1;
        pc.a.conj = s.conj_out ? 2 : 0;
        pc.a.tw = tw;
        pc.a.scale = 1.0f;
        pc.in_role = ROLE_SCRATCH;
        pc.out_role = s.out_role;
        pc.grid = dim3((N1 + kr->C - 1) / kr->C, N2 * s.batch);
        out.push_back(pc);
        if (r2c) {
            Pass p3;
            p3.type = PASS_R2C_FIXUP;
            p3.a.rtw = res.rtw;
            p3.out_role = s.out_role;
            p3.M = M;
            p3.dist = s.out_dist;
            p3.batch = s.batch;
            p3.full = s.epilogue == EPI_R2C_FULL;
            out.push_back(p3);
        }
        return true;
    }

    // Four-step: M = N1 * N2, x[n1*N2 + n2], X[k1 + N1*k2].
    const unsigned N1 = 1u << (lg / 2), N2 = M / N1;
    if (N2 > kMaxTile) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "transform length %u exceeds the two-pass limit", M);
        return false;
    }
    if (s.batch > 65535) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "batch %u too large for multi-pass lengths", s.batch);
        return false;
    }
    const TileKernel *kc = find_tile((int)N1, ACROSS, ACROSS);
    const TileKernel *kr = find_tile((int)N2, ALONG, ACROSS);
    if (!kc || !kr) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "no four-step kernels for %u x %u", N1, N2);
        return false;
    }
    if (!dry) {
        res.scratch_bytes = (size_t)M * s.batch * sizeof(float2);
        if (!cuda_ok(cudaMalloc(&res.scratch, res.scratch_bytes), "cudaMalloc(scratch)"))
            return false;
        if (use_twiddle_table(kc) && !upload_twlo(N1, kc->C, M, res.twlo))
            return false;
    }
    Pass p1;
    p1.k = kc;
    p1.a.in_stride = N2;
    p1.a.in_dist = 1;
    p1.a.in_batch = s.in_dist;
    p1.a.out_stride = N2;
    p1.a.out_dist = 1;
    p1.a.out_batch = M;
    p1.a.ntrans = N2;
    p1.a.conj = s.conj_in ? 1 : 0;
    p1.a.prologue = s.prologue;
    p1.a.half = s.half;
    p1.a.epilogue = EPI_TWIDDLE;
    p1.a.tw = tw;
    p1.a.rtw = res.rtw;
    p1.a.mirror_len = M;
    p1.a.mirror_ldist = 1;
    p1.a.scale = s.scale;
    p1.a.tw_scale = 2.0f / (float)M;
    p1.a.tw_mask = M - 1;
    p1.a.tw_lo = use_twiddle_table(kc) ? res.twlo : nullptr;
    p1.a.tw_colpow = use_colpow(kc) ? 1 : 0;
    p1.in_role = s.in_role;
    p1.in2_role = s.in2_role;
    p1.a.conj2 = s.conj2;
    p1.out_role = ROLE_SCRATCH;
    p1.grid = dim3((N2 + kc->C - 1) / kc->C, s.batch);
    out.push_back(p1);

    Pass p2;
    p2.k = kr;
    p2.a.in_stride = 1;
    p2.a.in_dist = N2;
    p2.a.in_batch = M;
    p2.a.out_stride = N1;
    p2.a.out_dist = 1;
    p2.a.out_batch = s.out_dist;
    p2.a.ntrans = N1;
    p2.a.conj = s.conj_out ? 2 : 0;
    p2.a.prologue = PRO_PLAIN;
    p2.a.epilogue = EPI_PLAIN;
    p2.a.tw = tw;
    p2.in_role = ROLE_SCRATCH;
    p2.out_role = s.out_role;
    p2.grid = dim3((N1 + kr->C - 1) / kr->C, s.batch);
    out.push_back(p2);

    if (r2c) {
        Pass p3;
        p3.type = PASS_R2C_FIXUP;
        p3.a.rtw = res.rtw;
        p3.out_role = s.out_role;
        p3.M = M;
        p3.dist = s.out_dist;
        p3.batch = s.batch;
        p3.full = s.epilogue == EPI_R2C_FULL;
        out.push_back(p3);
    }
    return true;
}

// Lazily allocated device staging for host-memory arguments.
struct Staging {
    void *in = nullptr, *out = nullptr, *in2 = nullptr;
    size_t in_bytes = 0, out_bytes = 0, in2_bytes = 0;
    void release()
    {
        cudaFree(in);
        cudaFree(out);
        cudaFree(in2);
        in = out = in2 = nullptr;
        in_bytes = out_bytes = in2_bytes = 0;
    }
};

bool ensure(void *&p, size_t &have, size_t need)
{
    if (have >= need && p)
        return true;
    cudaFree(p);
    p = nullptr;
    have = 0;
    if (!cuda_ok(cudaMalloc(&p, need ? need : 16), "cudaMalloc(staging)"))
        return false;
    have = need;
    return true;
}

}  // namespace

// ================================================================== 1D

enum Kind1D { K_C2C = 0, K_R2C = 1, K_C2R = 2 };

struct mufft_plan_1d {
    int device = -1;
    int kind = K_C2C;
    unsigned N = 0, M = 0;
    int direction = MUFFT_FORWARD;
    unsigned flags = 0;
    unsigned batch = 1;
    size_t in_elem = 8, out_elem = 8;    // bytes per input / output element
    size_t in_count = 0, out_count = 0;  // elements read / written per transform
    size_t idist = 0, odist = 0;         // elements between transforms
    std::vector<Pass> passes;
    PlanResources res;
    Staging stage;
    cudaStream_t stream = nullptr;
    bool uses_in2 = false;

    size_t in_total() const { return ((size_t)(batch - 1) * idist + in_count) * in_elem; }
    size_t out_total() const { return ((size_t)(batch - 1) * odist + out_count) * out_elem; }
};

namespace {

void destroy_1d(mufft_plan_1d *pl)
{
    if (!pl)
        return;
    if (pl->device >= 0) {
        DeviceGuard g(pl->device);
        pl->res.release();
        pl->stage.release();
        if (pl->stream)
            cudaStreamDestroy(pl->stream);
    }
    delete pl;
}

// ------------------------------------------------------------ autotune cache
//
// Remembered schedule choices per plan shape, filled by the autotuner
// (mufft_gb_autotune_1d, or plan creation with MUFFT_GB_FLAG_AUTOTUNE) or
// loaded from a file, and applied when a plan of that shape is created.
struct TuneKey {
    int kind;
    unsigned N, batch, flags;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(kind, N, batch, flags) < std::tie(o.kind, o.N, o.batch, o.flags);
    }
};
constexpr unsigned kTuneFlagMask = MUFFT_FLAG_FULL_R2C | MUFFT_FLAG_ZERO_PAD_UPPER_HALF;
std::mutex g_tune_mu;
std::map<TuneKey, PlanOptions> g_tune;

bool tune_lookup(int kind, unsigned N, unsigned batch, unsigned flags, PlanOptions *o)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(TuneKey{kind, N, batch, flags & kTuneFlagMask});
    if (it == g_tune.end())
        return false;
    *o = it->second;
    return true;
}

bool autotune_run(int kind, unsigned N, int direction, unsigned flags, unsigned batch, PlanOptions *best,
                  std::string *report);

// prologue_override: PRO_MUL / PRO_MUL_C2R for convolution output plans.
mufft_plan_1d *create_1d(int kind, unsigned N, int direction, unsigned flags, unsigned batch,
                         size_t idist, size_t odist, int prologue_override, bool dry,
                         std::string *desc, bool conj2 = false)
{
    t_err = 0;
    if (!is_pow2(N) || N == 1) {
        set_error(MUFFT_GB_ERR_INVALID, "N=%u is not a power of two >= 2", N);
        return nullptr;
    }
    if (kind == K_C2C && direction != MUFFT_FORWARD && direction != MUFFT_INVERSE) {
        set_error(MUFFT_GB_ERR_INVALID, "direction must be MUFFT_FORWARD or MUFFT_INVERSE");
        return nullptr;
    }
    if (kind != K_C2C && N < 4) {
        // the inner complex transform would have length 1 (fft.c:478-481 via :628-631)
        set_error(MUFFT_GB_ERR_INVALID, "real transforms need N >= 4");
        return nullptr;
    }
    if (batch == 0) {
        set_error(MUFFT_GB_ERR_INVALID, "batch must be >= 1");
        return nullptr;
    }
    const bool autotune = (flags & MUFFT_GB_FLAG_AUTOTUNE) != 0;
    flags &= ~MUFFT_GB_FLAG_AUTOTUNE;
    const bool zp = (flags & MUFFT_FLAG_ZERO_PAD_UPPER_HALF) != 0;
    const bool full = (flags & MUFFT_FLAG_FULL_R2C) != 0;
    const int split_limbs =
        (flags & MUFFT_GB_FLAG_SPLIT_BF16X3) ? 3 : ((flags & MUFFT_GB_FLAG_SPLIT_BF16X2) ? 2 : 0);
    if (split_limbs && (kind != K_C2C || (N != 256 && N != 4096) || zp || prologue_override >= 0)) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED,
                  "split-precision transforms are c2c of N = 256 or 4096 without zero padding");
        return nullptr;
    }

    mufft_plan_1d *pl = new mufft_plan_1d();
    pl->kind = kind;
    pl->N = N;
    pl->M = kind == K_C2C ? N : N / 2;
    pl->direction = kind == K_C2C ? direction : (kind == K_R2C ? MUFFT_FORWARD : MUFFT_INVERSE);
    pl->flags = flags;
    pl->batch = batch;
    const unsigned M = pl->M;

    FftSpec s;
    s.M = M;
    s.batch = batch;
    switch (kind) {
    case K_C2C:
        pl->in_elem = pl->out_elem = 8;
        pl->in_count = zp ? N / 2 : N;
        pl->out_count = N;
        s.epilogue = EPI_PLAIN;
        s.conj_in = s.conj_out = direction == MUFFT_INVERSE;
        break;
    case K_R2C:
        pl->in_elem = 4;
        pl->out_elem = 8;
        pl->in_count = zp ? N / 2 : N;
        pl->out_count = full ? N : N / 2 + 1;
        s.epilogue = full ? EPI_R2C_FULL : EPI_R2C;
        break;
    case K_C2R:
        pl->in_elem = 8;
        pl->out_elem = 4;
        pl->in_count = N / 2 + 1;
        pl->out_count = N;
        s.prologue = PRO_C2R;
        s.conj_in = s.conj_out = 1;
        break;
    }
    s.half = zp;
    if (prologue_override >= 0) {
        s.prologue = prologue_override;
        s.in2_role = ROLE_IN2;
        s.conj2 = conj2 ? 1 : 0;
        pl->uses_in2 = true;
    }
    // r2c input of N reals is read as M complex pairs.
    pl->idist = idist ? idist : (kind == K_R2C ? (zp ? N / 2 : N) : pl->in_count);
    pl->odist = odist ? odist : pl->out_count;
    if ((kind == K_R2C && (pl->idist & 1)) || (kind == K_C2R && (pl->odist & 1))) {
        set_error(MUFFT_GB_ERR_INVALID, "real-valued batch distances must be even");
        delete pl;
        return nullptr;
    }
    if (pl->idist < pl->in_count || pl->odist < pl->out_count) {
        set_error(MUFFT_GB_ERR_INVALID, "batch distance smaller than one transform");
        delete pl;
        return nullptr;
    }
    s.in_dist = kind == K_R2C ? (long long)pl->idist / 2 : (long long)pl->idist;
    s.out_dist = kind == K_C2R ? (long long)pl->odist / 2 : (long long)pl->odist;

    const float2 *tw = nullptr;
    if (!dry) {
        int dev;
        if (!device_prepare(&dev)) {
            delete pl;
            return nullptr;
        }
        pl->device = dev;
        tw = g_dev[dev].tw;
        if (kind != K_C2C) {
            pl->res.rtw = upload(r2c_twiddles(kind == K_R2C ? MUFFT_FORWARD : MUFFT_INVERSE, M));
            if (!pl->res.rtw) {
                destroy_1d(pl);
                return nullptr;
            }
        }
        if (!cuda_ok(cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking), "cudaStreamCreate")) {
            destroy_1d(pl);
            return nullptr;
        }
    }
    if (prologue_override >= 0 && kind == K_C2C)
        s.scale = 1.0f / (float)N;
    if (prologue_override >= 0 && kind == K_C2R)
        s.scale = 1.0f / (float)N;
    if (split_limbs) {
        Pass p;
        p.type = PASS_SPLIT;
        p.sp.in_dist = s.in_dist;
        p.sp.out_dist = s.out_dist;
        p.sp.ntrans = batch;
        p.sp.conj = direction == MUFFT_INVERSE ? 1 : 0;
        p.sp_stages = N == 256 ? 2 : 3;
        p.sp_limbs = split_limbs;
        p.sp_engine = g_split_engine.load();
        const unsigned per_cta = kSplitPoints / N;
        p.sp_grid = (batch + per_cta - 1) / per_cta;
        if (p.sp_engine == 0) {
            // persistent: two CTAs per SM (152 SMs on GB300 when no device is queried)
            int sms = 152;
            if (!dry)
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, pl->device);
            p.sp_grid = std::min(p.sp_grid, 2u * (unsigned)sms);
        }
        if (!dry) {
            const std::vector<unsigned> af = split_afrag_table();
            if (!cuda_ok(cudaMalloc(&pl->res.afrag, af.size() * sizeof(unsigned)), "cudaMalloc(split table)") ||
                !cuda_ok(cudaMemcpy(pl->res.afrag, af.data(), af.size() * sizeof(unsigned), cudaMemcpyHostToDevice),
                         "cudaMemcpy(split table)") ||
                !(pl->res.sptw = upload(split_twiddle_table())) ||
                !cuda_ok(cudaFuncSetAttribute(split_kernel(p.sp_stages, split_limbs),
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)split_smem_bytes()),
                         "cudaFuncSetAttribute(split)")) {
                destroy_1d(pl);
                return nullptr;
            }
            const std::vector<unsigned short> bf = split_umma_bfrag_table();
            if (!cuda_ok(cudaMalloc(&pl->res.bfrag, bf.size() * 2), "cudaMalloc(split table)") ||
                !cuda_ok(cudaMemcpy(pl->res.bfrag, bf.data(), bf.size() * 2, cudaMemcpyHostToDevice),
                         "cudaMemcpy(split table)") ||
                !cuda_ok(cudaMalloc(&pl->res.err, sizeof(int)), "cudaMalloc(error flag)") ||
                !cuda_ok(cudaMemset(pl->res.err, 0, sizeof(int)), "cudaMemset(error flag)") ||
                !cuda_ok(cudaFuncSetAttribute(split_umma_kernel(p.sp_stages, split_limbs),
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)split_umma_smem_bytes()),
                         "cudaFuncSetAttribute(split tcgen05)")) {
                destroy_1d(pl);
                return nullptr;
            }
            p.sp.afrag = pl->res.afrag;
            p.sp.tw = pl->res.sptw;
            p.sp.bfrag = pl->res.bfrag;
            p.sp.err = pl->res.err;
        }
        pl->passes.push_back(p);
    } else {
        // remembered (or, with MUFFT_GB_FLAG_AUTOTUNE, freshly tuned) schedule
        // choices apply unless the plan is being built with explicit ones
        PlanOptions tuned;
        const PlanOptions *prev = t_opts;
        if (!t_opts) {
            bool have = tune_lookup(kind, N, batch, flags, &tuned);
            if (!have && autotune && !dry) {
                have = autotune_run(kind, N, direction, flags, batch, &tuned, nullptr);
                t_err = 0;
            }
            if (have)
                t_opts = &tuned;
        }
        const bool built = build_fft_passes(s, tw, pl->res, dry, pl->passes) &&
                           attach_tma(pl->passes, pl->res, dry, pl->device) &&
                           attach_stream(pl->passes, dry, pl->device) &&
                           attach_occupancy(pl->passes, dry, pl->device);
        t_opts = prev;
        if (!built) {
            destroy_1d(pl);
            return nullptr;
        }
    }
    if (desc)
        *desc = describe(pl->passes);
    if (dry) {
        delete pl;
        return nullptr;
    }
    return pl;
}

// Runs a 1D plan; `sync` selects the fft.h semantics (any memory, blocking).
int exec_1d(mufft_plan_1d *pl, void *out, const void *in, const void *in2, cudaStream_t st, bool sync)
{
    if (!pl || !out || !in || (pl->uses_in2 && !in2)) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan or buffer");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(pl->device);
    const bool hin = !is_device_accessible(in);
    const bool hin2 = pl->uses_in2 && !is_device_accessible(in2);
    const bool hout = !is_device_accessible(out);
    if (!sync && (hin || hin2 || hout)) {
        set_error(MUFFT_GB_ERR_HOST_POINTER, "asynchronous execute needs device-accessible buffers");
        return MUFFT_GB_ERR_HOST_POINTER;
    }
    if (sync)
        st = pl->stream;
    Buffers b{in, out, in2, pl->res.scratch};
    if (hin) {
        if (!ensure(pl->stage.in, pl->stage.in_bytes, pl->in_total()))
            return t_err;
        if (!cuda_ok(cudaMemcpyAsync(pl->stage.in, in, pl->in_total(), cudaMemcpyDefault, st), "H2D copy"))
            return t_err;
        b.in = pl->stage.in;
    }
    if (hin2) {
        if (!ensure(pl->stage.in2, pl->stage.in2_bytes, pl->in_total()))
            return t_err;
        if (!cuda_ok(cudaMemcpyAsync(pl->stage.in2, in2, pl->in_total(), cudaMemcpyDefault, st), "H2D copy"))
            return t_err;
        b.in2 = pl->stage.in2;
    }
    if (hout) {
        if (!ensure(pl->stage.out, pl->stage.out_bytes, pl->out_total()))
            return t_err;
        b.out = pl->stage.out;
    }
    if (!cuda_ok(run_passes(pl->passes, b, st), "kernel launch"))
        return t_err;
    if (hout && !cuda_ok(cudaMemcpyAsync(out, b.out, pl->out_total(), cudaMemcpyDefault, st), "D2H copy"))
        return t_err;
    if (sync && !cuda_ok(cudaStreamSynchronize(st), "execute"))
        return t_err;
    if (sync && pl->res.err) {
        int e = 0;
        if (cuda_ok(cudaMemcpy(&e, pl->res.err, sizeof(int), cudaMemcpyDeviceToHost), "error flag") && e) {
            set_error(MUFFT_GB_ERR_UNSUPPORTED, "a bounded wait in a persistent kernel timed out");
            cudaMemset(pl->res.err, 0, sizeof(int));
            return t_err;
        }
    }
    return MUFFT_GB_OK;
}

std::string describe_options(const PlanOptions &o)
{
    std::string d;
    char b[160];
    snprintf(b, sizeof(b), "levels=%d twiddle=%d fused=%d tma=%d", o.levels, o.twiddle, o.fused, o.tma);
    d = b;
    for (const TileKernel &k : o.tiles) {
        snprintf(b, sizeof(b), " tile(L=%d %s/%s C=%d R=%d Q=%d)", k.L, k.lmap ? "across" : "along",
                 k.smap ? "across" : "along", k.C, k.R, k.Q);
        d += b;
    }
    return d;
}

// Times the candidate schedules of one plan shape on the current device and
// remembers the fastest.  Coordinate descent: the pass structure (levels,
// twiddle scheme, fused last passes) with default tiles first, then each
// tile role of the winner over its compiled variants.  Candidates run on
// zero-filled scratch buffers; each time is the best of three groups of
// back-to-back executes, measured with CUDA events.
bool autotune_run(int kind, unsigned N, int direction, unsigned flags, unsigned batch, PlanOptions *best,
                  std::string *report)
{
    const size_t bytes = (size_t)N * batch * sizeof(float2) + 256;
    void *din = nullptr, *dout = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&] {
        if (e0)
            cudaEventDestroy(e0);
        if (e1)
            cudaEventDestroy(e1);
        if (st)
            cudaStreamDestroy(st);
        cudaFree(din);
        cudaFree(dout);
    };
    if (!cuda_ok(cudaMalloc(&din, bytes), "cudaMalloc(autotune)") ||
        !cuda_ok(cudaMalloc(&dout, bytes), "cudaMalloc(autotune)") ||
        !cuda_ok(cudaMemset(din, 0, bytes), "cudaMemset(autotune)") ||
        !cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") || !cuda_ok(cudaEventCreate(&e1), "cudaEventCreate")) {
        cleanup();
        return false;
    }
    const size_t points = (size_t)N * batch;
    const int reps = (int)std::max<size_t>(3, std::min<size_t>(20, ((size_t)1 << 26) / std::max<size_t>(points, 1)));
    auto measure = [&](const PlanOptions &o, std::vector<TileKernel> *roles) -> double {
        const PlanOptions *prev = t_opts;
        t_opts = &o;
        mufft_plan_1d *pl = create_1d(kind, N, direction, flags, batch, 0, 0, -1, false, nullptr);
        t_opts = prev;
        if (!pl) {
            t_err = 0;
            return INFINITY;
        }
        if (roles) {
            roles->clear();
            for (const Pass &p : pl->passes) {
                if (p.type != PASS_TILE)
                    continue;
                bool seen = false;
                for (const TileKernel &r : *roles)
                    seen |= r.L == p.k->L && r.lmap == p.k->lmap && r.smap == p.k->smap;
                if (!seen)
                    roles->push_back(*p.k);
            }
        }
        double ms = INFINITY;
        bool ok = true;
        for (int w = 0; w < 2 && ok; w++)
            ok = exec_1d(pl, dout, din, nullptr, st, false) == MUFFT_GB_OK;
        for (int g = 0; g < 3 && ok; g++) {
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && ok; r++)
                ok = exec_1d(pl, dout, din, nullptr, st, false) == MUFFT_GB_OK;
            cudaEventRecord(e1, st);
            float t = 0.f;
            ok = ok && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess;
            if (ok)
                ms = std::min(ms, (double)t / reps);
        }
        destroy_1d(pl);
        if (!ok) {
            cudaGetLastError();
            t_err = 0;
            return INFINITY;
        }
        if (report) {
            char b[64];
            snprintf(b, sizeof(b), "%.4f ms  ", ms);
            *report += b + describe_options(o) + "\n";
        }
        return ms;
    };
    PlanOptions cur;
    double cur_ms = measure(cur, nullptr);
    const unsigned M = kind == K_C2C ? N : N / 2;
    if (M <= (unsigned)kMaxSinglePass) {
        for (const TileKernel &k : tile_table()) {
            if (k.L != (int)M || k.lmap != ALONG || k.smap != ALONG)
                continue;
            PlanOptions o;
            o.tiles = {k};
            const double t = measure(o, nullptr);
            if (t < cur_ms) {
                cur = o;
                cur_ms = t;
            }
        }
    } else {
        const unsigned lg = ilog2u(M);
        for (int lv = 2; lv <= 3; lv++)
            for (int tw = 0; tw <= 2; tw++)
                for (int fu = 0; fu <= ((lv == 3 && lg >= 20) ? 1 : 0); fu++) {
                    PlanOptions o;
                    o.levels = lv;
                    o.twiddle = tw;
                    o.fused = fu;
                    const double t = measure(o, nullptr);
                    if (t < cur_ms) {
                        cur = o;
                        cur_ms = t;
                    }
                }
        for (int tm = 0; tm <= 2; tm++) {
            PlanOptions o = cur;
            o.tma = tm;
            const double t = measure(o, nullptr);
            if (t < cur_ms) {
                cur = o;
                cur_ms = t;
            }
        }
        std::vector<TileKernel> roles;
        cur_ms = std::min(cur_ms, measure(cur, &roles));
        for (const TileKernel &role : roles) {
            for (const TileKernel &k : tile_table()) {
                if (k.L != role.L || k.lmap != role.lmap || k.smap != role.smap)
                    continue;
                PlanOptions o = cur;
                bool replaced = false;
                for (TileKernel &t : o.tiles)
                    if (t.L == k.L && t.lmap == k.lmap && t.smap == k.smap) {
                        t = k;
                        replaced = true;
                    }
                if (!replaced)
                    o.tiles.push_back(k);
                const double t = measure(o, nullptr);
                if (t < cur_ms) {
                    cur = o;
                    cur_ms = t;
                }
            }
        }
    }
    cleanup();
    if (!std::isfinite(cur_ms)) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "no schedule of this shape ran");
        return false;
    }
    if (report) {
        char b[64];
        snprintf(b, sizeof(b), "best %.4f ms  ", cur_ms);
        *report += b + describe_options(cur) + "\n";
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune[TuneKey{kind, N, batch, flags & kTuneFlagMask}] = cur;
    }
    *best = cur;
    return true;
}

}  // namespace

extern "C" {

mufft_plan_1d *mufft_create_plan_1d_c2c(unsigned N, int direction, unsigned flags)
{
    return create_1d(K_C2C, N, direction, flags, 1, 0, 0, -1, false, nullptr);
}

mufft_plan_1d *mufft_create_plan_1d_r2c(unsigned N, unsigned flags)
{
    return create_1d(K_R2C, N, MUFFT_FORWARD, flags, 1, 0, 0, -1, false, nullptr);
}

mufft_plan_1d *mufft_create_plan_1d_c2r(unsigned N, unsigned flags)
{
    return create_1d(K_C2R, N, MUFFT_INVERSE, flags, 1, 0, 0, -1, false, nullptr);
}

mufft_plan_1d *mufft_gb_create_plan_1d_c2c_batched(unsigned N, int direction, unsigned flags,
                                                   unsigned batch, size_t idist, size_t odist)
{
    return create_1d(K_C2C, N, direction, flags, batch, idist, odist, -1, false, nullptr);
}

mufft_plan_1d *mufft_gb_create_plan_1d_r2c_batched(unsigned N, unsigned flags, unsigned batch,
                                                   size_t idist, size_t odist)
{
    return create_1d(K_R2C, N, MUFFT_FORWARD, flags, batch, idist, odist, -1, false, nullptr);
}

mufft_plan_1d *mufft_gb_create_plan_1d_c2r_batched(unsigned N, unsigned flags, unsigned batch,
                                                   size_t idist, size_t odist)
{
    return create_1d(K_C2R, N, MUFFT_INVERSE, flags, batch, idist, odist, -1, false, nullptr);
}

void mufft_execute_plan_1d(mufft_plan_1d *plan, void *MUFFT_RESTRICT output, const void *MUFFT_RESTRICT input)
{
    exec_1d(plan, output, input, nullptr, nullptr, true);
}

int mufft_gb_execute_plan_1d_launches_async(mufft_plan_1d *plan, void *output, const void *input,
                                            unsigned first, unsigned count, void *stream)
{
    if (!plan || plan->uses_in2 || !is_device_accessible(output) || !is_device_accessible(input)) {
        set_error(MUFFT_GB_ERR_INVALID, "needs a single-input plan and device buffers");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(plan->device);
    Buffers b{input, output, nullptr, plan->res.scratch};
    if (!cuda_ok(run_passes(plan->passes, b, (cudaStream_t)stream, first, count), "kernel launch"))
        return t_err;
    return MUFFT_GB_OK;
}

int mufft_gb_execute_plan_1d_async(mufft_plan_1d *plan, void *output, const void *input, void *stream)
{
    if (plan && plan->uses_in2) {
        set_error(MUFFT_GB_ERR_INVALID, "plan needs two inputs");
        return MUFFT_GB_ERR_INVALID;
    }
    return exec_1d(plan, output, input, nullptr, (cudaStream_t)stream, false);
}

void mufft_free_plan_1d(mufft_plan_1d *plan) { destroy_1d(plan); }

unsigned mufft_gb_plan_1d_launches(const mufft_plan_1d *plan) { return plan ? (unsigned)plan->passes.size() : 0; }

int mufft_gb_plan_1d_describe(const mufft_plan_1d *plan, char *buf, size_t size)
{
    if (!plan || !buf || !size)
        return MUFFT_GB_ERR_INVALID;
    snprintf(buf, size, "%s", describe(plan->passes).c_str());
    return MUFFT_GB_OK;
}

// Describes the launches a 1D plan would use, without a GPU.  kind: 0 c2c,
// 1 r2c, 2 c2r.
int mufft_gb_describe_schedule_1d(unsigned N, int kind, int direction, unsigned flags, unsigned batch,
                                  char *buf, size_t size)
{
    std::string d;
    if (kind < 0 || kind > 2) {
        set_error(MUFFT_GB_ERR_INVALID, "kind must be 0, 1 or 2");
        return MUFFT_GB_ERR_INVALID;
    }
    t_err = 0;
    create_1d(kind, N, direction, flags, batch, 0, 0, -1, true, &d);
    if (t_err)
        return t_err;
    if (buf && size)
        snprintf(buf, size, "%s", d.c_str());
    return MUFFT_GB_OK;
}

}  // extern "C"

// ================================================================ conv

struct mufft_plan_conv {
    unsigned N = 0;
    unsigned method = 0;
    size_t block_size = 0;
    mufft_plan_1d *in_plan[2] = {nullptr, nullptr};
    mufft_plan_1d *out_plan = nullptr;
    // adjoints (mufft_gb_conv_adjoint_*), made on first use
    int device = -1;
    mufft_plan_1d *adj_fwd = nullptr;        // gradient of the output -> spectrum (full length)
    mufft_plan_1d *adj_mul = nullptr;        // x conj(second spectrum), 1/N, inverse
    mufft_plan_1d *adj_fwd_batch = nullptr;  // the forward transform over a chunk of gradients
    unsigned adj_chunk = 0;
    size_t adj_dist = 0;
    mufft_plan_1d *adj_c2r = nullptr;        // N/2 + 1 bins -> N reals
    float2 *adj_spec = nullptr;              // spectra of the gradients
    size_t adj_spec_bytes = 0;
    float2 *adj_acc = nullptr;               // N/2 + 1 bins of the filter gradient
    // batched forms (mufft_gb_execute_conv_output_batched, mufft_gb_conv_adjoint):
    // plans over a chunk of signals and over the ragged last chunk
    struct BatchPlan {
        mufft_plan_1d *pl = nullptr;
        unsigned batch = 0;
        size_t idist = 0, odist = 0;
    };
    BatchPlan out_b[2], fwd_b[2], inv_b[2];
};

extern "C" {

mufft_plan_conv *mufft_create_plan_conv(unsigned N, unsigned flags, unsigned method)
{
    t_err = 0;
    if (!is_pow2(N) || N == 1) {
        set_error(MUFFT_GB_ERR_INVALID, "N=%u is not a power of two >= 2", N);
        return nullptr;
    }
    mufft_plan_conv *c = new mufft_plan_conv();
    c->N = N;
    c->method = method;
    const unsigned zp0 = (method & MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST) ? MUFFT_FLAG_ZERO_PAD_UPPER_HALF : 0;
    const unsigned zp1 = (method & MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND) ? MUFFT_FLAG_ZERO_PAD_UPPER_HALF : 0;
    const unsigned base = flags & ~(unsigned)MUFFT_FLAG_ZERO_PAD_UPPER_HALF;
    if ((method & 1u) == MUFFT_CONV_METHOD_FLAG_STEREO_MONO) {
        // fft.c:593-599
        c->block_size = (size_t)N * 8;
        c->in_plan[0] = create_1d(K_C2C, N, MUFFT_FORWARD, flags | zp0, 1, 0, 0, -1, false, nullptr);
        c->in_plan[1] = create_1d(K_R2C, N, MUFFT_FORWARD, flags | zp1 | MUFFT_FLAG_FULL_R2C, 1, 0, 0, -1, false, nullptr);
        c->out_plan = create_1d(K_C2C, N, MUFFT_INVERSE, base, 1, 0, 0, PRO_MUL, false, nullptr);
    } else {
        // fft.c:585-591
        c->block_size = (size_t)(N / 2 + 4) * 8;
        c->in_plan[0] = create_1d(K_R2C, N, MUFFT_FORWARD, flags | zp0, 1, 0, 0, -1, false, nullptr);
        c->in_plan[1] = create_1d(K_R2C, N, MUFFT_FORWARD, flags | zp1, 1, 0, 0, -1, false, nullptr);
        c->out_plan = create_1d(K_C2R, N, MUFFT_INVERSE, base, 1, 0, 0, PRO_MUL_C2R, false, nullptr);
    }
    if (!c->in_plan[0] || !c->in_plan[1] || !c->out_plan) {
        mufft_free_plan_conv(c);
        return nullptr;
    }
    c->device = c->out_plan->device;
    return c;
}

void mufft_execute_conv_input(mufft_plan_conv *plan, unsigned block, void *output, const void *input)
{
    if (!plan) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan");
        return;
    }
    exec_1d(plan->in_plan[block ? 1 : 0], output, input, nullptr, nullptr, true);
}

size_t mufft_conv_get_transformed_block_size(mufft_plan_conv *plan) { return plan ? plan->block_size : 0; }

void mufft_execute_conv_output(mufft_plan_conv *plan, void *output, const void *input_first,
                               const void *input_second)
{
    if (!plan) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan");
        return;
    }
    exec_1d(plan->out_plan, output, input_first, input_second, nullptr, true);
}

int mufft_gb_execute_conv_input_async(mufft_plan_conv *plan, unsigned block, void *output,
                                      const void *input, void *stream)
{
    if (!plan) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan");
        return MUFFT_GB_ERR_INVALID;
    }
    return exec_1d(plan->in_plan[block ? 1 : 0], output, input, nullptr, (cudaStream_t)stream, false);
}

int mufft_gb_execute_conv_output_async(mufft_plan_conv *plan, void *output, const void *input_first,
                                       const void *input_second, void *stream)
{
    if (!plan) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan");
        return MUFFT_GB_ERR_INVALID;
    }
    return exec_1d(plan->out_plan, output, input_first, input_second, (cudaStream_t)stream, false);
}

void mufft_free_plan_conv(mufft_plan_conv *plan)
{
    if (!plan)
        return;
    for (int i = 0; i < 2; i++) {
        destroy_1d(plan->out_b[i].pl);
        destroy_1d(plan->fwd_b[i].pl);
        destroy_1d(plan->inv_b[i].pl);
    }
    destroy_1d(plan->in_plan[0]);
    destroy_1d(plan->in_plan[1]);
    destroy_1d(plan->out_plan);
    destroy_1d(plan->adj_fwd);
    destroy_1d(plan->adj_mul);
    destroy_1d(plan->adj_fwd_batch);
    destroy_1d(plan->adj_c2r);
    if (plan->device >= 0) {
        DeviceGuard g(plan->device);
        cudaFree(plan->adj_spec);
        cudaFree(plan->adj_acc);
    }
    delete plan;
}

}  // extern "C"

// ============================================================ conv adjoint
//
// For out = (1/N) IFFT(FFT(first) . FFT(second)) (fft.c:794-809) and an
// upstream gradient G_out of `out`:
//   d/d first  = (1/N) IFFT(FFT(G_out) . conj(FFT(second)))
//   d/d second = Re (1/N) IFFT(sum_b FFT(G_out_b) . conj(FFT(first_b)))
// (complex gradients in the d/dRe + i d/dIm convention; the second block is
// real in both conv methods).

namespace {

bool conv_stereo(const mufft_plan_conv *c) { return (c->method & 1u) == MUFFT_CONV_METHOD_FLAG_STEREO_MONO; }

// Spectrum bins of one gradient block: N/2 + 1 (mono r2c) or N (stereo).
size_t conv_bins(const mufft_plan_conv *c) { return conv_stereo(c) ? c->N : c->N / 2 + 1; }

bool conv_adj_spec(mufft_plan_conv *c, size_t bytes)
{
    if (c->adj_spec_bytes >= bytes)
        return true;
    cudaFree(c->adj_spec);
    c->adj_spec = nullptr;
    c->adj_spec_bytes = 0;
    if (!cuda_ok(cudaMalloc(&c->adj_spec, bytes), "cudaMalloc(adjoint spectra)"))
        return false;
    c->adj_spec_bytes = bytes;
    return true;
}

}  // namespace

extern "C" {

int mufft_gb_conv_adjoint_input(mufft_plan_conv *plan, void *grad_input, const void *grad_output,
                                const void *second_spectrum, void *stream)
{
    if (!plan || !grad_input || !grad_output || !second_spectrum) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan or buffer");
        return MUFFT_GB_ERR_INVALID;
    }
    t_err = 0;
    DeviceGuard g(plan->device);
    const bool stereo = conv_stereo(plan);
    const unsigned N = plan->N;
    if (!plan->adj_fwd)
        plan->adj_fwd = create_1d(stereo ? K_C2C : K_R2C, N, MUFFT_FORWARD, 0, 1, 0, 0, -1, false, nullptr);
    if (!plan->adj_mul)
        plan->adj_mul = create_1d(stereo ? K_C2C : K_C2R, N, MUFFT_INVERSE, 0, 1, 0, 0,
                                  stereo ? PRO_MUL : PRO_MUL_C2R, false, nullptr, true);
    if (!plan->adj_fwd || !plan->adj_mul)
        return t_err ? t_err : MUFFT_GB_ERR_ALLOC;
    if (!conv_adj_spec(plan, conv_bins(plan) * sizeof(float2)))
        return t_err;
    const cudaStream_t st = (cudaStream_t)stream;
    int rc = exec_1d(plan->adj_fwd, plan->adj_spec, grad_output, nullptr, st, false);
    if (rc != MUFFT_GB_OK)
        return rc;
    return exec_1d(plan->adj_mul, grad_input, plan->adj_spec, second_spectrum, st, false);
}

int mufft_gb_conv_adjoint_filter(mufft_plan_conv *plan, float *grad_filter, const void *grad_outputs,
                                 size_t output_dist, const void *first_spectra, size_t spectrum_dist,
                                 unsigned batch, void *stream)
{
    if (!plan || !grad_filter || !grad_outputs || !first_spectra || batch == 0) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan or buffer, or empty batch");
        return MUFFT_GB_ERR_INVALID;
    }
    t_err = 0;
    const bool stereo = conv_stereo(plan);
    const unsigned N = plan->N;
    const size_t bins = conv_bins(plan);
    if (output_dist < N || (!stereo && (output_dist & 1)) || spectrum_dist < bins) {
        set_error(MUFFT_GB_ERR_INVALID, "batch distances smaller than one block");
        return MUFFT_GB_ERR_INVALID;
    }
    if (!is_device_accessible(grad_filter) || !is_device_accessible(grad_outputs) ||
        !is_device_accessible(first_spectra)) {
        set_error(MUFFT_GB_ERR_HOST_POINTER, "the adjoint needs device-accessible buffers");
        return MUFFT_GB_ERR_HOST_POINTER;
    }
    DeviceGuard g(plan->device);
    // Gradients are transformed in chunks whose spectra stay within 256 MiB.
    size_t chunk = ((size_t)256 << 20) / (bins * sizeof(float2));
    chunk = chunk < 1 ? 1 : chunk;
    chunk = chunk > batch ? batch : chunk;
    if (!plan->adj_fwd_batch || plan->adj_chunk != chunk || plan->adj_dist != output_dist) {
        destroy_1d(plan->adj_fwd_batch);
        plan->adj_fwd_batch = create_1d(stereo ? K_C2C : K_R2C, N, MUFFT_FORWARD, 0, (unsigned)chunk,
                                        output_dist, bins, -1, false, nullptr);
        plan->adj_chunk = plan->adj_fwd_batch ? (unsigned)chunk : 0;
        plan->adj_dist = output_dist;
    }
    if (!plan->adj_c2r)
        plan->adj_c2r = create_1d(K_C2R, N, MUFFT_INVERSE, 0, 1, 0, 0, -1, false, nullptr);
    if (!plan->adj_fwd_batch || !plan->adj_c2r)
        return t_err ? t_err : MUFFT_GB_ERR_ALLOC;
    if (!conv_adj_spec(plan, chunk * bins * sizeof(float2)))
        return t_err;
    if (!plan->adj_acc && !cuda_ok(cudaMalloc(&plan->adj_acc, (N / 2 + 1) * sizeof(float2)), "cudaMalloc"))
        return t_err;
    const cudaStream_t st = (cudaStream_t)stream;
    const size_t elem = stereo ? sizeof(float2) : sizeof(float);  // one sample of a gradient block
    const float2 *A = (const float2 *)first_spectra;
    for (size_t b0 = 0; b0 < batch; b0 += chunk) {
        const size_t n = batch - b0 < chunk ? batch - b0 : chunk;
        const char *src = (const char *)grad_outputs + b0 * output_dist * elem;
        if (n == chunk) {
            const int rc = exec_1d(plan->adj_fwd_batch, plan->adj_spec, src, nullptr, st, false);
            if (rc != MUFFT_GB_OK)
                return rc;
        } else {
            // ragged last chunk: one transform at a time with the single-block plan
            if (!plan->adj_fwd)
                plan->adj_fwd = create_1d(stereo ? K_C2C : K_R2C, N, MUFFT_FORWARD, 0, 1, 0, 0, -1, false, nullptr);
            if (!plan->adj_fwd)
                return t_err ? t_err : MUFFT_GB_ERR_ALLOC;
            for (size_t i = 0; i < n; i++) {
                const int rc = exec_1d(plan->adj_fwd, plan->adj_spec + i * bins, src + i * output_dist * elem,
                                       nullptr, st, false);
                if (rc != MUFFT_GB_OK)
                    return rc;
            }
        }
        if (!cuda_ok(launch_adjoint_filter_reduce(plan->adj_acc, plan->adj_spec, (long long)bins,
                                                  A + b0 * spectrum_dist, (long long)spectrum_dist, (unsigned)n,
                                                  N, stereo ? 1 : 0, 1.0f / (float)N, b0 > 0 ? 1 : 0, st),
                     "adjoint reduce"))
            return t_err;
    }
    return exec_1d(plan->adj_c2r, grad_filter, plan->adj_acc, nullptr, st, false);
}

}  // extern "C"

namespace {

// A batched plan of `batch` transforms, remade when its shape changes.  With
// a prologue (spectral multiply) the second spectrum is one for the whole
// batch (in2_bcast).
mufft_plan_1d *conv_batch_plan(mufft_plan_conv::BatchPlan &bp, int kind, unsigned N, int direction, unsigned batch,
                               size_t idist, size_t odist, int prologue, bool conj2)
{
    if (bp.pl && bp.batch == batch && bp.idist == idist && bp.odist == odist)
        return bp.pl;
    destroy_1d(bp.pl);
    bp = mufft_plan_conv::BatchPlan{};
    mufft_plan_1d *pl = create_1d(kind, N, direction, 0, batch, idist, odist, prologue, false, nullptr, conj2);
    if (!pl)
        return nullptr;
    for (Pass &p : pl->passes)
        if (p.type == PASS_TILE && p.in2_role != ROLE_NONE)
            p.a.in2_bcast = pl->passes.size() == 1 ? 2 : 1;  // batch by transform index / by grid row
    bp.pl = pl;
    bp.batch = batch;
    bp.idist = idist;
    bp.odist = odist;
    return pl;
}

// Signals per chunk of a batched convolution call: spectra (and multi-pass
// scratch) of a chunk stay within 256 MiB.
size_t conv_chunk(const mufft_plan_conv *c, unsigned batch)
{
    size_t chunk = ((size_t)256 << 20) / (conv_bins(c) * sizeof(float2));
    chunk = chunk < 1 ? 1 : chunk;
    return chunk > batch ? batch : chunk;
}

}  // namespace

extern "C" {

int mufft_gb_execute_conv_output_batched(mufft_plan_conv *plan, void *outputs, size_t output_dist,
                                         const void *first_spectra, size_t spectrum_dist, const void *second_spectrum,
                                         unsigned batch, void *stream)
{
    if (!plan || !outputs || !first_spectra || !second_spectrum || batch == 0) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan or buffer, or empty batch");
        return MUFFT_GB_ERR_INVALID;
    }
    t_err = 0;
    const bool stereo = conv_stereo(plan);
    const unsigned N = plan->N;
    if (output_dist < N || (!stereo && (output_dist & 1)) || spectrum_dist < conv_bins(plan)) {
        set_error(MUFFT_GB_ERR_INVALID, "batch distances smaller than one block");
        return MUFFT_GB_ERR_INVALID;
    }
    if (!is_device_accessible(outputs) || !is_device_accessible(first_spectra) ||
        !is_device_accessible(second_spectrum)) {
        set_error(MUFFT_GB_ERR_HOST_POINTER, "batched convolution needs device-accessible buffers");
        return MUFFT_GB_ERR_HOST_POINTER;
    }
    DeviceGuard g(plan->device);
    const cudaStream_t st = (cudaStream_t)stream;
    const size_t chunk = conv_chunk(plan, batch);
    const size_t elem = stereo ? sizeof(float2) : sizeof(float);
    for (size_t b0 = 0; b0 < batch; b0 += chunk) {
        const size_t n = batch - b0 < chunk ? batch - b0 : chunk;
        mufft_plan_1d *pl = conv_batch_plan(plan->out_b[n == chunk ? 0 : 1], stereo ? K_C2C : K_C2R, N,
                                            MUFFT_INVERSE, (unsigned)n, spectrum_dist, output_dist,
                                            stereo ? PRO_MUL : PRO_MUL_C2R, false);
        if (!pl)
            return t_err ? t_err : MUFFT_GB_ERR_ALLOC;
        const int rc = exec_1d(pl, (char *)outputs + b0 * output_dist * elem,
                               (const float2 *)first_spectra + b0 * spectrum_dist, second_spectrum, st, false);
        if (rc != MUFFT_GB_OK)
            return rc;
    }
    return MUFFT_GB_OK;
}

int mufft_gb_conv_adjoint(mufft_plan_conv *plan, float *grad_filter, void *grad_inputs, size_t input_dist,
                          const void *grad_outputs, size_t output_dist, const void *first_spectra,
                          size_t spectrum_dist, const void *second_spectrum, unsigned batch, void *stream)
{
    if (!plan || !grad_outputs || batch == 0 || (!grad_filter && !grad_inputs) || (grad_filter && !first_spectra) ||
        (grad_inputs && !second_spectrum)) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan or buffer, nothing to compute, or empty batch");
        return MUFFT_GB_ERR_INVALID;
    }
    t_err = 0;
    const bool stereo = conv_stereo(plan);
    const unsigned N = plan->N;
    const size_t bins = conv_bins(plan);
    if (output_dist < N || (!stereo && (output_dist & 1)) || (grad_filter && spectrum_dist < bins) ||
        (grad_inputs && (input_dist < N || (!stereo && (input_dist & 1))))) {
        set_error(MUFFT_GB_ERR_INVALID, "batch distances smaller than one block");
        return MUFFT_GB_ERR_INVALID;
    }
    if (!is_device_accessible(grad_outputs) || (grad_filter && (!is_device_accessible(grad_filter) ||
                                                                !is_device_accessible(first_spectra))) ||
        (grad_inputs && (!is_device_accessible(grad_inputs) || !is_device_accessible(second_spectrum)))) {
        set_error(MUFFT_GB_ERR_HOST_POINTER, "the adjoint needs device-accessible buffers");
        return MUFFT_GB_ERR_HOST_POINTER;
    }
    DeviceGuard g(plan->device);
    const cudaStream_t st = (cudaStream_t)stream;
    const size_t chunk = conv_chunk(plan, batch);
    const size_t elem = stereo ? sizeof(float2) : sizeof(float);
    if (!conv_adj_spec(plan, chunk * bins * sizeof(float2)))
        return t_err;
    if (grad_filter) {
        if (!plan->adj_c2r)
            plan->adj_c2r = create_1d(K_C2R, N, MUFFT_INVERSE, 0, 1, 0, 0, -1, false, nullptr);
        if (!plan->adj_c2r)
            return t_err ? t_err : MUFFT_GB_ERR_ALLOC;
        if (!plan->adj_acc && !cuda_ok(cudaMalloc(&plan->adj_acc, (N / 2 + 1) * sizeof(float2)), "cudaMalloc"))
            return t_err;
    }
    const float2 *A = (const float2 *)first_spectra;
    for (size_t b0 = 0; b0 < batch; b0 += chunk) {
        const size_t n = batch - b0 < chunk ? batch - b0 : chunk;
        const int w = n == chunk ? 0 : 1;
        // one forward transform of each output gradient serves both gradients
        mufft_plan_1d *fwd = conv_batch_plan(plan->fwd_b[w], stereo ? K_C2C : K_R2C, N, MUFFT_FORWARD, (unsigned)n,
                                             output_dist, bins, -1, false);
        if (!fwd)
            return t_err ? t_err : MUFFT_GB_ERR_ALLOC;
        int rc = exec_1d(fwd, plan->adj_spec, (const char *)grad_outputs + b0 * output_dist * elem, nullptr, st, false);
        if (rc != MUFFT_GB_OK)
            return rc;
        if (grad_filter &&
            !cuda_ok(launch_adjoint_filter_reduce(plan->adj_acc, plan->adj_spec, (long long)bins,
                                                  A + b0 * spectrum_dist, (long long)spectrum_dist, (unsigned)n, N,
                                                  stereo ? 1 : 0, 1.0f / (float)N, b0 > 0 ? 1 : 0, st),
                     "adjoint reduce"))
            return t_err;
        if (grad_inputs) {
            mufft_plan_1d *inv = conv_batch_plan(plan->inv_b[w], stereo ? K_C2C : K_C2R, N, MUFFT_INVERSE,
                                                 (unsigned)n, bins, input_dist, stereo ? PRO_MUL : PRO_MUL_C2R, true);
            if (!inv)
                return t_err ? t_err : MUFFT_GB_ERR_ALLOC;
            rc = exec_1d(inv, (char *)grad_inputs + b0 * input_dist * elem, plan->adj_spec, second_spectrum, st, false);
            if (rc != MUFFT_GB_OK)
                return rc;
        }
    }
    if (grad_filter)
        return exec_1d(plan->adj_c2r, grad_filter, plan->adj_acc, nullptr, st, false);
    return MUFFT_GB_OK;
}

}  // extern "C"

// ======================================================= convolve func

namespace {

// Element-wise multiply for mufft_get_convolve_func: any memory, blocking.
void gpu_convolve(void *output, const void *a, const void *b, float normalization, unsigned samples)
{
    if (!output || !a || !b) {
        set_error(MUFFT_GB_ERR_INVALID, "null buffer");
        return;
    }
    int dev;
    if (!device_prepare(&dev))
        return;
    const size_t bytes = (size_t)samples * sizeof(float2);
    const bool ha = !is_device_accessible(a), hb = !is_device_accessible(b), ho = !is_device_accessible(output);
    float2 *da = (float2 *)a, *db = (float2 *)b, *dout = (float2 *)output;
    float2 *tmp = nullptr;
    if (ha || hb || ho) {
        if (!cuda_ok(cudaMalloc(&tmp, 3 * bytes + 16), "cudaMalloc(convolve)"))
            return;
        if (ha) {
            da = tmp;
            cudaMemcpy(da, a, bytes, cudaMemcpyDefault);
        }
        if (hb) {
            db = tmp + samples;
            cudaMemcpy(db, b, bytes, cudaMemcpyDefault);
        }
        if (ho)
            dout = tmp + 2 * (size_t)samples;
    }
    if (cuda_ok(launch_spectral_multiply(dout, da, db, normalization, samples, nullptr), "convolve")) {
        if (ho)
            cuda_ok(cudaMemcpy(output, dout, bytes, cudaMemcpyDefault), "D2H copy");
        else
            cuda_ok(cudaDeviceSynchronize(), "convolve");
    }
    cudaFree(tmp);
}

}  // namespace

extern "C" mufft_convolve_func mufft_get_convolve_func(unsigned flags)
{
    (void)flags;
    return &gpu_convolve;
}

// ================================================================ ragged conv

struct mufft_gb_conv_batch {
    int device = -1;
    unsigned count = 0;
    RaggedReq *d_reqs = nullptr;
    RaggedTask *d_tasks = nullptr;
    unsigned *d_next = nullptr;      // [0] dequeue counter, [1..] per split request completed tasks
    int *d_err = nullptr;
    float2 *d_scratch = nullptr;
    float2 *d_rtw = nullptr;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned grid = 0;
    unsigned split_lg = 16;          // requests of 2^split_lg complex points and more run as phase tasks
    unsigned class_lg = 14;          // requests of 2^class_lg points and more run as class pipelines
    unsigned small_grid = 0;         // persistent CTAs when class pipelines run beside them (0: all SMs)
    std::vector<RaggedReq> sorted;   // longest first (host copy)
    RaggedArgs args{};
    size_t smem = 0;
    ClassEntry *d_class = nullptr;
    const float2 **d_tab = nullptr;  // group tasks' buffer tables
    std::vector<cudaStream_t> class_streams;
    std::vector<cudaEvent_t> class_events;
    cudaEvent_t fork_event = nullptr;
    int sms = 0;
};

namespace {

void destroy_conv_batch(mufft_gb_conv_batch *b)
{
    if (!b)
        return;
    if (b->device >= 0) {
        DeviceGuard g(b->device);
        if (b->exec)
            cudaGraphExecDestroy(b->exec);
        if (b->graph)
            cudaGraphDestroy(b->graph);
        if (b->capture)
            cudaStreamDestroy(b->capture);
        for (cudaStream_t cs : b->class_streams)
            cudaStreamDestroy(cs);
        for (cudaEvent_t ev : b->class_events)
            cudaEventDestroy(ev);
        if (b->fork_event)
            cudaEventDestroy(b->fork_event);
        cudaFree(b->d_class);
        cudaFree(b->d_tab);
        cudaFree(b->d_reqs);
        cudaFree(b->d_tasks);
        cudaFree(b->d_err);
        cudaFree(b->d_next);
        cudaFree(b->d_scratch);
        cudaFree(b->d_rtw);
    }
    delete b;
}

// Split size of ragged batches created afterwards (log2 of complex points;
// 17: no request is split), set with mufft_gb_set_conv_split.  Default 2^16:
// on the 512-request mix (2^8..2^16 points) splitting the 65536-point
// requests took the batch from 0.19 to 0.177 ms, splitting 32768 and 16384
// as well cost more in task overhead than it gained (0.226, 0.259 ms).
std::atomic<unsigned> g_conv_split_lg{16};
// Requests of 2^g_conv_class_lg complex points and more run as class
// pipelines (ordinary batched launches per size class; 17: none).  Default
// 2^14: on the 512-request mix the batch went from 0.177 ms (split tasks for
// 65536) to 0.152 / 0.148 / 0.146 ms with classes from 65536 / 32768 / 16384.
std::atomic<unsigned> g_conv_class_lg{14};

// Task list for a split size, uploaded with the request table, and the graph
// (counter resets + the persistent launch) that replays it.
// Launches of one class pipeline (five four-step phases over the class's
// requests) on `st`.
bool enqueue_class(mufft_gb_conv_batch *b, unsigned lg, bool stereo, bool zp, const ClassEntry *tab, unsigned K,
                   cudaStream_t st)
{
    const int L1 = lg == 16 ? 256 : 128, L2 = lg == 14 ? 128 : 256, L = L1 * L2;
    const ClassTile ct = class_column_tile(L1), rt = class_row_tile(L2), rmt = class_row_mul_tile(L2);
    TileArgs base{};
    base.tw = g_dev[b->device].tw;
    base.scale = 1.0f;
    base.tw_scale = 2.0f / (float)L;
    base.tw_mask = (unsigned)(L - 1);
    TileArgs cols = base, rows = base;
    cols.in_stride = cols.out_stride = L2;
    cols.in_dist = cols.out_dist = 1;
    cols.ntrans = (unsigned)L2;
    rows.in_stride = rows.out_stride = 1;
    rows.in_dist = rows.out_dist = L2;
    rows.ntrans = (unsigned)L1;
    TileArgs ph[5] = {cols, rows, base, rows, cols};
    ph[0].half = zp ? 1 : 0;
    ph[0].epilogue = EPI_TWIDDLE;
    ph[0].tw_colpow = 1;
    ph[3].conj = 1;
    ph[3].epilogue = EPI_TWIDDLE;
    ph[4].conj = 2;
    if (stereo) {
        // the spectral multiply rides in F2's epilogue: X[k1 + L1*k2] * H[k1 + L1*k2] / L
        ph[1].in2_dist = 1;
        ph[1].in2_stride = L1;
        ph[1].scale = 1.0f / (float)L;
    }
    for (int phase = 0; phase < 5; phase++) {
        cudaError_t e;
        if (phase == 2 && stereo)
            continue;
        if (phase == 2) {
            // mono: r2c pairs, multiply, c2r pairs (stereo classes did it in F2)
            const unsigned l1 = ilog2u((unsigned)L1), l2 = ilog2u((unsigned)L2);
            float scale = 1.0f / (float)(2 * L);
            const float2 *rf = b->d_rtw + b->args.rtw_off[lg], *ri = rf + L;
            void *args[] = {(void *)&tab, (void *)&l1, (void *)&l2, &scale, (void *)&rf, (void *)&ri};
            e = cudaLaunchKernel(class_multiply_fn(), dim3((unsigned)(L1 / 32), (unsigned)(L2 / 64), K), dim3(256), args,
                                 0, st);
        } else {
            const ClassTile &t = (phase == 0 || phase == 4) ? ct : (phase == 1 && stereo ? rmt : rt);
            const unsigned tiles = (phase == 0 || phase == 4) ? (unsigned)(L2 / t.C) : (unsigned)(L1 / t.C);
            int phase_ = phase;
            void *args[] = {&ph[phase], (void *)&tab, &phase_};
            e = cudaLaunchKernel(t.fn, dim3(tiles, K), dim3(t.threads), args, t.smem, st);
        }
        if (!cuda_ok(e, "class launch"))
            return false;
    }
    return true;
}

bool conv_batch_build(mufft_gb_conv_batch *b, unsigned split_lg, unsigned class_lg, unsigned small_grid)
{
    DeviceGuard g(b->device);
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    cudaFree(b->d_tasks);
    cudaFree(b->d_next);
    b->d_tasks = nullptr;
    b->d_next = nullptr;
    b->split_lg = split_lg;
    b->class_lg = class_lg;
    b->small_grid = small_grid;
    cudaFree(b->d_class);
    b->d_class = nullptr;
    cudaFree(b->d_tab);
    b->d_tab = nullptr;
    std::vector<RaggedReq> reqs = b->sorted;
    std::vector<unsigned> split_ids, whole_ids;
    // class pipelines: (lg, stereo, zero pad) -> requests
    std::map<std::tuple<unsigned, unsigned, unsigned>, std::vector<unsigned>> classes;
    unsigned nsplit = 0;
    for (unsigned i = 0; i < reqs.size(); i++) {
        if (reqs[i].lg >= class_lg && reqs[i].lg >= kRaggedMinSplitLg) {
            classes[std::make_tuple(reqs[i].lg, reqs[i].stereo, reqs[i].zero_pad)].push_back(i);
            continue;
        }
        reqs[i].split = reqs[i].lg >= split_lg && reqs[i].lg >= kRaggedMinSplitLg ? 1 : 0;
        if (reqs[i].split) {
            reqs[i].counter = 1 + nsplit++;
            split_ids.push_back(i);
        } else {
            whole_ids.push_back(i);
        }
    }
    // Whole requests of sizes whose tile holds several transforms run in
    // groups: up to that many requests of one class per task, their buffers
    // in tables.  Work items keep the longest-first order.
    std::vector<RaggedTask> whole;
    std::vector<const float2 *> tab;
    {
        std::map<std::tuple<unsigned, unsigned, unsigned>, std::vector<unsigned>> open;
        auto flush = [&](std::vector<unsigned> &g) {
            RaggedTask t{g[0], kRaggedGroupTask, (unsigned short)g.size(), 0, (unsigned)tab.size()};
            for (unsigned r : g)
                tab.push_back(reqs[r].in);
            for (unsigned r : g)
                tab.push_back(reqs[r].h);
            for (unsigned r : g)
                tab.push_back(reqs[r].out);
            for (unsigned r : g)
                tab.push_back(reqs[r].spec);
            whole.push_back(t);
            g.clear();
        };
        for (unsigned r : whole_ids) {
            const unsigned gs = ragged_group_size(reqs[r].lg);
            if (gs <= 1) {
                whole.push_back(RaggedTask{r, 0, 0, 0, 0});
                continue;
            }
            std::vector<unsigned> &g = open[std::make_tuple(reqs[r].lg, reqs[r].stereo, reqs[r].zero_pad)];
            g.push_back(r);
            if (g.size() == gs)
                flush(g);
        }
        for (auto &kv : open)
            if (!kv.second.empty())
                flush(kv.second);
        // longest first (requests arrive sorted by cost; a group costs about one member)
        std::stable_sort(whole.begin(), whole.end(), [&](const RaggedTask &x, const RaggedTask &y) {
            return reqs[x.req].lg > reqs[y.req].lg;
        });
    }
    // phase-major over split requests, with whole requests (longest first) in between
    std::vector<RaggedTask> tasks;
    size_t w = 0;
    for (unsigned phase = 0; phase < 5; phase++) {
        for (unsigned r : split_ids) {
            unsigned before = 0;
            for (unsigned p = 0; p < phase; p++)
                before += ragged_phase_tasks(reqs[r].lg, p);
            for (unsigned t = 0; t < ragged_phase_tasks(reqs[r].lg, phase); t++)
                tasks.push_back(RaggedTask{r, (unsigned short)phase, (unsigned short)t, before, 0});
        }
        const size_t take = phase == 4 ? whole.size() - w : (whole.size() - w) / (5 - phase);
        for (size_t k = 0; k < take; k++, w++)
            tasks.push_back(whole[w]);
    }
    b->args.count = (unsigned)tasks.size();
    std::vector<ClassEntry> entries;
    std::vector<std::tuple<unsigned, unsigned, unsigned, size_t, unsigned>> class_list;  // lg, stereo, zp, offset, K
    for (const auto &kv : classes) {
        class_list.push_back(std::make_tuple(std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first),
                                             entries.size(), (unsigned)kv.second.size()));
        for (unsigned r : kv.second)
            entries.push_back(ClassEntry{reqs[r].in, reqs[r].h, reqs[r].out, reqs[r].spec});
    }
    while (b->class_streams.size() < class_list.size()) {
        cudaStream_t cs;
        cudaEvent_t ev;
        if (!cuda_ok(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate") ||
            !cuda_ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate"))
            return false;
        b->class_streams.push_back(cs);
        b->class_events.push_back(ev);
    }
    if (!b->fork_event && !cuda_ok(cudaEventCreateWithFlags(&b->fork_event, cudaEventDisableTiming), "cudaEventCreate"))
        return false;
    if (!entries.empty() &&
        (!cuda_ok(cudaMalloc(&b->d_class, entries.size() * sizeof(ClassEntry)), "cudaMalloc(classes)") ||
         !cuda_ok(cudaMemcpy(b->d_class, entries.data(), entries.size() * sizeof(ClassEntry), cudaMemcpyHostToDevice),
                  "cudaMemcpy(classes)")))
        return false;
    if (!tab.empty() &&
        (!cuda_ok(cudaMalloc(&b->d_tab, tab.size() * sizeof(float2 *)), "cudaMalloc(group tables)") ||
         !cuda_ok(cudaMemcpy(b->d_tab, tab.data(), tab.size() * sizeof(float2 *), cudaMemcpyHostToDevice),
                  "cudaMemcpy(group tables)")))
        return false;
    b->args.tab = b->d_tab;
    if (!cuda_ok(cudaMalloc(&b->d_tasks, std::max<size_t>(1, tasks.size()) * sizeof(RaggedTask)), "cudaMalloc(tasks)") ||
        !cuda_ok(cudaMemcpy(b->d_tasks, tasks.data(), tasks.size() * sizeof(RaggedTask), cudaMemcpyHostToDevice),
                 "cudaMemcpy(tasks)") ||
        !cuda_ok(cudaMemcpy(b->d_reqs, reqs.data(), reqs.size() * sizeof(RaggedReq), cudaMemcpyHostToDevice),
                 "cudaMemcpy(requests)") ||
        !cuda_ok(cudaMalloc(&b->d_next, (1 + nsplit) * sizeof(unsigned)), "cudaMalloc(counters)"))
        return false;
    b->args.tasks = b->d_tasks;
    b->args.next = b->d_next;
    b->args.counters = b->d_next;
    b->args.err = b->d_err;
    unsigned grid = std::min<unsigned>(b->grid, (unsigned)tasks.size());
    if (!class_list.empty() && small_grid)
        grid = std::min(grid, small_grid);
    void *kargs[] = {&b->args};
    bool ok = cuda_ok(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "capture") &&
              cuda_ok(cudaMemsetAsync(b->d_next, 0, (1 + nsplit) * sizeof(unsigned), b->capture), "cudaMemsetAsync");
    // class pipelines on parallel branches, then the persistent kernel for the rest
    if (ok && !class_list.empty())
        ok = cuda_ok(cudaEventRecord(b->fork_event, b->capture), "fork");
    for (size_t c = 0; ok && c < class_list.size(); c++) {
        const auto &cl = class_list[c];
        ok = cuda_ok(cudaStreamWaitEvent(b->class_streams[c], b->fork_event, 0), "fork") &&
             enqueue_class(b, std::get<0>(cl), std::get<1>(cl) != 0, std::get<2>(cl) != 0, b->d_class + std::get<3>(cl),
                           std::get<4>(cl), b->class_streams[c]) &&
             cuda_ok(cudaEventRecord(b->class_events[c], b->class_streams[c]), "join");
    }
    if (ok && !tasks.empty())
        ok = cuda_ok(cudaLaunchKernel(conv_ragged_fn(), dim3(grid), dim3(conv_ragged_threads()), kargs, b->smem,
                                      b->capture),
                     "kernel launch");
    for (size_t c = 0; ok && c < class_list.size(); c++)
        ok = cuda_ok(cudaStreamWaitEvent(b->capture, b->class_events[c], 0), "join");
    cudaGraph_t gr = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b->capture, &gr);
    if (!ok || !cuda_ok(ce, "capture") || !cuda_ok(cudaGraphInstantiate(&b->exec, gr, 0), "cudaGraphInstantiate")) {
        if (gr)
            cudaGraphDestroy(gr);
        return false;
    }
    b->graph = gr;
    return true;
}

}  // namespace

extern "C" {

mufft_gb_conv_batch *mufft_gb_create_conv_batch(const mufft_gb_conv_request *requests, unsigned count,
                                                unsigned flags)
{
    t_err = 0;
    if (!requests || count == 0) {
        set_error(MUFFT_GB_ERR_INVALID, "no requests");
        return nullptr;
    }
    std::vector<RaggedReq> reqs(count);
    std::vector<unsigned long long> cost(count);
    bool need[17] = {};
    size_t scratch_elems = 0;
    std::vector<size_t> spec_off(count);
    for (unsigned i = 0; i < count; i++) {
        const mufft_gb_conv_request &r = requests[i];
        const bool stereo = (r.method & 1u) == MUFFT_CONV_METHOD_FLAG_STEREO_MONO;
        if (!is_pow2(r.N) || !r.input || !r.filter || !r.output) {
            set_error(MUFFT_GB_ERR_INVALID, "request %u: N must be a power of two and buffers non-null", i);
            return nullptr;
        }
        const unsigned L = stereo ? r.N : r.N / 2;
        const unsigned lg = ilog2u(L);
        if (L < 16 || L > 65536) {
            set_error(MUFFT_GB_ERR_UNSUPPORTED, "request %u: N=%u outside the ragged range", i, r.N);
            return nullptr;
        }
        RaggedReq &q = reqs[i];
        q.in = (const float2 *)r.input;
        q.h = (const float2 *)r.filter;
        q.out = (float2 *)r.output;
        q.scale = 1.0f / (float)r.N;
        q.lg = lg;
        q.stereo = stereo ? 1 : 0;
        q.zero_pad = (r.method & MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST) ? 1 : 0;
        need[lg] = true;
        cost[i] = (unsigned long long)L * lg;
        spec_off[i] = scratch_elems;
        scratch_elems += ((size_t)L + 1 + 31) & ~(size_t)31;  // 256-byte aligned slots
    }
    int dev;
    if (!device_prepare(&dev))
        return nullptr;
    mufft_gb_conv_batch *b = new mufft_gb_conv_batch();
    b->device = dev;
    b->count = count;
    RaggedArgs &args = b->args;
    // per-size r2c / c2r fix-up twiddles, FP64 then rounded (fft.c:441-455)
    std::vector<float2> rtw;
    for (unsigned lg = 0; lg <= 16; lg++) {
        args.rtw_off[lg] = (unsigned)rtw.size();
        if (!need[lg])
            continue;
        std::vector<float2> f = r2c_twiddles(MUFFT_FORWARD, 1u << lg), iv = r2c_twiddles(MUFFT_INVERSE, 1u << lg);
        rtw.insert(rtw.end(), f.begin(), f.end());
        rtw.insert(rtw.end(), iv.begin(), iv.end());
    }
    if (rtw.empty())
        rtw.push_back(make_float2(0.f, 0.f));
    b->d_rtw = upload(rtw);
    if (!b->d_rtw || !cuda_ok(cudaMalloc(&b->d_scratch, scratch_elems * sizeof(float2)), "cudaMalloc(scratch)") ||
        !cuda_ok(cudaMalloc(&b->d_next, sizeof(unsigned)), "cudaMalloc(counter)") ||
        !cuda_ok(cudaMalloc(&b->d_reqs, count * sizeof(RaggedReq)), "cudaMalloc(requests)")) {
        destroy_conv_batch(b);
        return nullptr;
    }
    // longest first (LPT), so the largest requests start at once
    std::vector<unsigned> order(count);
    for (unsigned i = 0; i < count; i++)
        order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](unsigned x, unsigned y) { return cost[x] > cost[y]; });
    b->sorted.resize(count);
    for (unsigned i = 0; i < count; i++) {
        b->sorted[i] = reqs[order[i]];
        b->sorted[i].spec = b->d_scratch + spec_off[order[i]];
    }
    b->smem = conv_ragged_smem();
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (!cuda_ok(cudaFuncSetAttribute(conv_ragged_fn(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem),
                 "cudaFuncSetAttribute") ||
        !cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, conv_ragged_fn(), conv_ragged_threads(),
                                                               b->smem),
                 "occupancy") ||
        !cuda_ok(cudaMalloc(&b->d_err, sizeof(int)), "cudaMalloc(err)") ||
        !cuda_ok(cudaMemset(b->d_err, 0, sizeof(int)), "cudaMemset(err)") ||
        !cuda_ok(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), "cudaStreamCreate")) {
        destroy_conv_batch(b);
        return nullptr;
    }
    b->grid = (unsigned)(sms * std::max(per_sm, 1));
    b->sms = sms;
    b->args.reqs = b->d_reqs;
    b->args.tw = g_dev[dev].tw;
    b->args.rtw = b->d_rtw;
    unsigned best_lg = g_conv_split_lg.load(), best_class = g_conv_class_lg.load(), best_small = 0;
    if (flags & MUFFT_GB_FLAG_AUTOTUNE) {
        // time the batch with every split size (17: nothing split) and keep the fastest
        cudaEvent_t e0, e1;
        double best = INFINITY;
        bool ok = cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") && cuda_ok(cudaEventCreate(&e1), "cudaEventCreate");
        struct Cand {
            unsigned split_lg, class_lg, small_grid;
        };
        std::vector<Cand> cands;
        for (unsigned lg = kRaggedMinSplitLg; lg <= 17; lg++)
            cands.push_back(Cand{lg, 17, 0});
        for (unsigned cl = kRaggedMinSplitLg; cl <= 16; cl++)
            for (unsigned div : {1u, 2u, 4u})
                cands.push_back(Cand{17, cl, (unsigned)b->sms / div});
        Cand best_c{best_lg, g_conv_class_lg.load(), 0};
        for (const Cand &cd : cands) {
            if (!ok)
                break;
            if (!conv_batch_build(b, cd.split_lg, cd.class_lg, cd.small_grid)) {
                ok = false;
                break;
            }
            for (int wu = 0; wu < 2; wu++)
                cudaGraphLaunch(b->exec, b->capture);
            cudaEventRecord(e0, b->capture);
            for (int r = 0; r < 5; r++)
                cudaGraphLaunch(b->exec, b->capture);
            cudaEventRecord(e1, b->capture);
            float ms = 0.f;
            ok = cuda_ok(cudaEventSynchronize(e1), "autotune") && cuda_ok(cudaEventElapsedTime(&ms, e0, e1), "autotune");
            if (ok && ms < best) {
                best = ms;
                best_c = cd;
            }
        }
        best_lg = best_c.split_lg;
        best_class = best_c.class_lg;
        best_small = best_c.small_grid;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (!ok) {
            destroy_conv_batch(b);
            return nullptr;
        }
    }
    if (!conv_batch_build(b, best_lg, best_class, best_small)) {
        destroy_conv_batch(b);
        return nullptr;
    }
    return b;
}

int mufft_gb_execute_conv_batch(mufft_gb_conv_batch *batch, void *stream)
{
    if (!batch) {
        set_error(MUFFT_GB_ERR_INVALID, "null batch");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(batch->device);
    if (!cuda_ok(cudaGraphLaunch(batch->exec, (cudaStream_t)stream), "cudaGraphLaunch"))
        return t_err;
    return MUFFT_GB_OK;
}

int mufft_gb_conv_batch_status(mufft_gb_conv_batch *batch)
{
    if (!batch) {
        set_error(MUFFT_GB_ERR_INVALID, "null batch");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(batch->device);
    int e = 0;
    if (!cuda_ok(cudaDeviceSynchronize(), "synchronize") ||
        !cuda_ok(cudaMemcpy(&e, batch->d_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag"))
        return t_err;
    if (e) {
        cudaMemset(batch->d_err, 0, sizeof(int));
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "a bounded wait in the ragged batch timed out");
        return MUFFT_GB_ERR_UNSUPPORTED;
    }
    return MUFFT_GB_OK;
}

unsigned mufft_gb_conv_batch_split_size(const mufft_gb_conv_batch *batch)
{
    if (!batch || batch->split_lg >= 17 || batch->split_lg >= batch->class_lg)
        return 0u;
    return 1u << batch->split_lg;
}

unsigned mufft_gb_conv_batch_class_size(const mufft_gb_conv_batch *batch)
{
    return batch ? (batch->class_lg >= 17 ? 0u : 1u << batch->class_lg) : 0u;
}

void mufft_gb_free_conv_batch(mufft_gb_conv_batch *batch) { destroy_conv_batch(batch); }

}  // extern "C"

// ======================================================= streaming convolution

static std::atomic<unsigned> g_stream_ranges{0};
static std::atomic<int> g_stream_fused{1};

struct mufft_gb_stream_conv {
    int device = -1;
    unsigned block = 0, P = 0, nb = 0, pitch = 0;
    bool stereo = false;
    mufft_plan_1d *fwd = nullptr, *inv = nullptr;
    void *win = nullptr;      // 2 x block samples: previous block, then the caller's input
    float2 *xcur = nullptr;   // spectrum of the current window (nb bins)
    float2 *fdl = nullptr;    // P rows of `pitch` bins: spectra of the last P windows
    float2 *h = nullptr;      // P rows of `pitch` bins: filter-partition spectra
    float2 *y = nullptr;      // nb bins of the output spectrum
    void *ybuf = nullptr;     // 2 x block samples of the inverse; the output is the second half
    float2 *part = nullptr;   // G rows of `pitch` bins: partial sums of the multiply-accumulate
    unsigned G = 1;           // partition ranges per bin group
    int M = 0;                // nonzero: one fused launch per block, row tiles of M points
    int *err = nullptr;       // a bounded wait of the fused launch timed out
    UpolsBlockArgs block_args{};
    unsigned *counter = nullptr;  // [0] blocks processed, [1] CTA ticket, [2 + x] bin-group tickets
    size_t counter_bytes = 0;
    cudaStream_t capture = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

void destroy_stream_conv(mufft_gb_stream_conv *c)
{
    if (!c)
        return;
    destroy_1d(c->fwd);
    destroy_1d(c->inv);
    if (c->device >= 0) {
        DeviceGuard g(c->device);
        if (c->exec)
            cudaGraphExecDestroy(c->exec);
        if (c->capture)
            cudaStreamDestroy(c->capture);
        cudaFree(c->win);
        cudaFree(c->xcur);
        cudaFree(c->fdl);
        cudaFree(c->h);
        cudaFree(c->y);
        cudaFree(c->ybuf);
        cudaFree(c->part);
        cudaFree(c->counter);
        cudaFree(c->err);
    }
    delete c;
}

}  // namespace

extern "C" {

mufft_gb_stream_conv *mufft_gb_create_stream_conv(unsigned block, unsigned method, const float *filter, unsigned taps,
                                                  unsigned flags)
{
    t_err = 0;
    if (!is_pow2(block) || block < 2 || block > (1u << 23) || !filter || taps == 0) {
        set_error(MUFFT_GB_ERR_INVALID, "block must be a power of two in 2..2^23 and the filter non-empty");
        return nullptr;
    }
    const bool stereo = (method & 1u) == MUFFT_CONV_METHOD_FLAG_STEREO_MONO;
    const unsigned L = 2 * block;
    const unsigned P = (taps + block - 1) / block;
    const unsigned nb = stereo ? L : block + 1;
    const unsigned pitch = upols_pitch(nb);
    const unsigned tflags = flags & ~(unsigned)(MUFFT_FLAG_ZERO_PAD_UPPER_HALF | MUFFT_FLAG_FULL_R2C);
    mufft_gb_stream_conv *c = new mufft_gb_stream_conv();
    c->block = block;
    c->P = P;
    c->nb = nb;
    c->pitch = pitch;
    c->stereo = stereo;
    c->fwd = create_1d(stereo ? K_C2C : K_R2C, L, MUFFT_FORWARD, tflags, 1, 0, 0, -1, false, nullptr);
    c->inv = create_1d(stereo ? K_C2C : K_C2R, L, MUFFT_INVERSE, tflags, 1, 0, 0, -1, false, nullptr);
    if (!c->fwd || !c->inv) {
        destroy_stream_conv(c);
        return nullptr;
    }
    c->device = c->fwd->device;
    DeviceGuard g(c->device);
    const size_t sample = stereo ? sizeof(float2) : sizeof(float);
    // filter partitions: P zero-padded windows of L reals, transformed as one batch
    mufft_plan_1d *hp = create_1d(K_R2C, L, MUFFT_FORWARD, tflags | (stereo ? MUFFT_FLAG_FULL_R2C : 0), P,
                                  L, pitch, -1, false, nullptr);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const unsigned want_ranges = g_stream_ranges.load();
    // One launch per block when both transforms are one 256-thread row tile
    const unsigned M = stereo ? L : L / 2;
    auto row_tile = [M](const mufft_plan_1d *pl) {
        if (pl->passes.size() != 1)
            return false;
        const Pass &p = pl->passes[0];
        return p.type == PASS_TILE && p.k && !p.tk && !p.sk && p.smem_min == 0 && p.k->Q == 1 && p.k->R == 16 &&
               p.k->lmap == ALONG && p.k->smap == ALONG && p.k->L == (int)M && p.k->C * p.k->L == 4096 &&
               p.grid.x == 1 && p.grid.y == 1 && p.in_role == ROLE_IN && p.out_role == ROLE_OUT;
    };
    if (g_stream_fused.load() && upols_block_supported((int)M) && row_tile(c->fwd) && row_tile(c->inv)) {
        int per_sm = 0;
        if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, upols_block_fn((int)M), 256,
                                                                   upols_block_smem((int)M)),
                     "occupancy(stream convolution)")) {
            destroy_stream_conv(c);
            return nullptr;
        }
        c->M = (int)M;
        // partitions 1 .. P-1 over ranges (at least one range CTA per group:
        // it finishes the group); all CTAs resident at once
        const unsigned slots = (unsigned)std::max(2, sms * std::max(per_sm, 1));
        const unsigned max_g = std::max(1u, (slots - 1) / upols_groups(nb));
        c->G = std::max(1u, std::min({want_ranges ? want_ranges : max_g, max_g, std::max(P - 1, 1u)}));
    } else {
        c->G = want_ranges ? std::min(want_ranges, P) : upols_chunks(nb, P, sms);
    }
    c->counter_bytes = (c->M ? upols_block_tickets(upols_groups(nb)) : 2 + upols_groups(nb)) * sizeof(unsigned);
    float *hpad = nullptr;
    bool ok = hp && cuda_ok(cudaMalloc(&c->win, 2 * (size_t)block * sample), "cudaMalloc(window)") &&
              cuda_ok(cudaMalloc(&c->xcur, (size_t)nb * sizeof(float2)), "cudaMalloc(spectrum)") &&
              cuda_ok(cudaMalloc(&c->fdl, (size_t)P * pitch * sizeof(float2)), "cudaMalloc(delay line)") &&
              cuda_ok(cudaMalloc(&c->h, (size_t)P * pitch * sizeof(float2)), "cudaMalloc(filter spectra)") &&
              cuda_ok(cudaMemset(c->h, 0, (size_t)P * pitch * sizeof(float2)), "cudaMemset") &&
              cuda_ok(cudaMalloc(&c->y, (size_t)nb * sizeof(float2)), "cudaMalloc(output spectrum)") &&
              cuda_ok(cudaMalloc(&c->ybuf, 2 * (size_t)block * sample), "cudaMalloc(output)") &&
              cuda_ok(cudaMalloc(&c->part, (size_t)std::max(c->G, 1u) * pitch * sizeof(float2)),
                      "cudaMalloc(partials)") &&
              cuda_ok(cudaMalloc(&c->counter, c->counter_bytes), "cudaMalloc(counter)") &&
              cuda_ok(cudaMalloc(&c->err, sizeof(int)), "cudaMalloc(err)") &&
              cuda_ok(cudaMemset(c->err, 0, sizeof(int)), "cudaMemset") &&
              cuda_ok(cudaMalloc(&hpad, (size_t)P * L * sizeof(float)), "cudaMalloc(partitions)") &&
              cuda_ok(cudaMemset(hpad, 0, (size_t)P * L * sizeof(float)), "cudaMemset") &&
              cuda_ok(cudaMemset(c->win, 0, 2 * (size_t)block * sample), "cudaMemset") &&
              cuda_ok(cudaMemset(c->fdl, 0, (size_t)P * pitch * sizeof(float2)), "cudaMemset") &&
              cuda_ok(cudaMemset(c->counter, 0, c->counter_bytes), "cudaMemset");
    // partition p = filter[p*block .. (p+1)*block) at the start of window p
    for (unsigned p = 0; ok && p < P; p++) {
        const unsigned n = std::min(block, taps - p * block);
        ok = cuda_ok(cudaMemcpy(hpad + (size_t)p * L, filter + (size_t)p * block, n * sizeof(float), cudaMemcpyDefault),
                     "cudaMemcpy(filter)");
    }
    ok = ok && exec_1d(hp, c->h, hpad, nullptr, nullptr, false) == MUFFT_GB_OK &&
         cuda_ok(cudaDeviceSynchronize(), "filter spectra");
    destroy_1d(hp);
    cudaFree(hpad);
    if (!ok) {
        destroy_stream_conv(c);
        return nullptr;
    }
    // one block: spectrum of [previous, input], multiply-accumulate, inverse,
    // then the input becomes the previous block -- one fused launch, or a
    // graph of the separate launches
    if (c->M) {
        UpolsBlockArgs &a = c->block_args;
        a.fwd = c->fwd->passes[0].a;
        a.fwd.in = (const float2 *)c->win;
        a.fwd.out = c->xcur;
        a.fwd.in2 = nullptr;
        a.inv = c->inv->passes[0].a;
        a.inv_c2r_rows = (a.inv.prologue == PRO_C2R && a.inv.mirror_ldist == 0 && a.inv.mirror_len == (long long)M &&
                          !a.inv.half && a.inv.in_stride == 1)
                             ? 1
                             : 0;
        a.inv.in = c->y;
        a.inv.out = (float2 *)c->ybuf;
        a.inv.in2 = nullptr;
        a.xcur = c->xcur;
        a.fdl = c->fdl;
        a.h = c->h;
        a.part = c->part;
        a.y = c->y;
        a.win = (float4 *)c->win;
        a.half16 = (unsigned)((size_t)block * sample / 16);
        a.nb = nb;
        a.pitch = pitch;
        a.P = P;
        a.G = c->G;
        a.groups = upols_groups(nb);
        a.tickets = c->counter;
        a.err = c->err;
        a.s = 1.0f / (float)L;
        a.wait_polls = kUpolsWaitPolls;
        a.wait_skew = 0;
        return c;
    }
    cudaGraph_t gr = nullptr;
    ok = cuda_ok(cudaStreamCreateWithFlags(&c->capture, cudaStreamNonBlocking), "cudaStreamCreate") &&
         cuda_ok(cudaStreamBeginCapture(c->capture, cudaStreamCaptureModeThreadLocal), "capture");
    if (ok) {
        const bool body = exec_1d(c->fwd, c->xcur, c->win, nullptr, c->capture, false) == MUFFT_GB_OK &&
                          cuda_ok(launch_upols_mac(c->y, c->xcur, c->fdl, c->h, c->part, nb, P, c->G, c->counter,
                                                   1.0f / (float)L, c->capture),
                                  "multiply-accumulate") &&
                          exec_1d(c->inv, c->ybuf, c->y, nullptr, c->capture, false) == MUFFT_GB_OK &&
                          cuda_ok(cudaMemcpyAsync(c->win, (char *)c->win + (size_t)block * sample,
                                                  (size_t)block * sample, cudaMemcpyDeviceToDevice, c->capture),
                                  "window shift");
        const cudaError_t ce = cudaStreamEndCapture(c->capture, &gr);
        ok = body && cuda_ok(ce, "capture") && cuda_ok(cudaGraphInstantiate(&c->exec, gr, 0), "cudaGraphInstantiate");
        if (gr)
            cudaGraphDestroy(gr);
    }
    if (!ok) {
        destroy_stream_conv(c);
        return nullptr;
    }
    return c;
}

void *mufft_gb_stream_conv_input(mufft_gb_stream_conv *c)
{
    if (!c)
        return nullptr;
    return (char *)c->win + (size_t)c->block * (c->stereo ? sizeof(float2) : sizeof(float));
}

const void *mufft_gb_stream_conv_output(const mufft_gb_stream_conv *c)
{
    if (!c)
        return nullptr;
    return (const char *)c->ybuf + (size_t)c->block * (c->stereo ? sizeof(float2) : sizeof(float));
}

int mufft_gb_stream_conv_process(mufft_gb_stream_conv *c, void *stream)
{
    if (!c) {
        set_error(MUFFT_GB_ERR_INVALID, "null convolver");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(c->device);
    if (c->M) {
        // one kernel: launched directly (a graph launch adds latency)
        if (!cuda_ok(launch_upols_block(c->M, c->block_args, (cudaStream_t)stream), "block launch"))
            return t_err;
        return MUFFT_GB_OK;
    }
    if (!cuda_ok(cudaGraphLaunch(c->exec, (cudaStream_t)stream), "cudaGraphLaunch"))
        return t_err;
    return MUFFT_GB_OK;
}

int mufft_gb_stream_conv_reset(mufft_gb_stream_conv *c, void *stream)
{
    if (!c) {
        set_error(MUFFT_GB_ERR_INVALID, "null convolver");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(c->device);
    const cudaStream_t st = (cudaStream_t)stream;
    const size_t sample = c->stereo ? sizeof(float2) : sizeof(float);
    if (!cuda_ok(cudaMemsetAsync(c->win, 0, 2 * (size_t)c->block * sample, st), "reset") ||
        !cuda_ok(cudaMemsetAsync(c->fdl, 0, (size_t)c->P * c->pitch * sizeof(float2), st), "reset") ||
        !cuda_ok(cudaMemsetAsync(c->counter, 0, c->counter_bytes, st), "reset"))
        return t_err;
    return MUFFT_GB_OK;
}

void mufft_gb_free_stream_conv(mufft_gb_stream_conv *c) { destroy_stream_conv(c); }

int mufft_gb_set_stream_conv_ranges(unsigned ranges)
{
    if (ranges > (1u << 20)) {
        set_error(MUFFT_GB_ERR_INVALID, "at most 2^20 partition ranges");
        return MUFFT_GB_ERR_INVALID;
    }
    g_stream_ranges.store(ranges);
    return MUFFT_GB_OK;
}

unsigned mufft_gb_stream_conv_ranges(const mufft_gb_stream_conv *c) { return c ? c->G : 0u; }

int mufft_gb_set_stream_conv_fused(int enable)
{
    if (enable < 0 || enable > 1) {
        set_error(MUFFT_GB_ERR_INVALID, "enable must be 0 or 1");
        return MUFFT_GB_ERR_INVALID;
    }
    g_stream_fused.store(enable);
    return MUFFT_GB_OK;
}

int mufft_gb_stream_conv_fused(const mufft_gb_stream_conv *c) { return c && c->M ? 1 : 0; }

int mufft_gb_stream_conv_inject_timeout(mufft_gb_stream_conv *c, int enable)
{
    if (!c || enable < 0 || enable > 1) {
        set_error(MUFFT_GB_ERR_INVALID, "null convolver or enable not 0 / 1");
        return MUFFT_GB_ERR_INVALID;
    }
    if (!c->M) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "only one-launch blocks wait on other CTAs");
        return MUFFT_GB_ERR_UNSUPPORTED;
    }
    c->block_args.wait_skew = enable ? 1u : 0u;
    c->block_args.wait_polls = enable ? kUpolsInjectedWaitPolls : kUpolsWaitPolls;
    return MUFFT_GB_OK;
}

int mufft_gb_stream_conv_status(mufft_gb_stream_conv *c)
{
    if (!c) {
        set_error(MUFFT_GB_ERR_INVALID, "null convolver");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(c->device);
    int e = 0;
    if (!cuda_ok(cudaDeviceSynchronize(), "synchronize") ||
        !cuda_ok(cudaMemcpy(&e, c->err, sizeof(int), cudaMemcpyDeviceToHost), "error flag"))
        return t_err;
    if (e) {
        cudaMemset(c->err, 0, sizeof(int));
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "a bounded wait in the block launch timed out");
        return MUFFT_GB_ERR_UNSUPPORTED;
    }
    return MUFFT_GB_OK;
}

}  // extern "C"

// ================================================================== 2D

enum Kind2D { K2_C2C = 0, K2_R2C = 1, K2_C2R = 2 };

struct mufft_plan_2d {
    int device = -1;
    int kind = K2_C2C;
    unsigned Nx = 0, Ny = 0, Mx = 0;
    int direction = MUFFT_FORWARD;
    unsigned flags = 0;
    unsigned vertical_nx = 0;
    std::vector<Pass> passes;
    PlanResources res;
    Staging stage;
    cudaStream_t stream = nullptr;
    // bytes moved for host buffers: rows x width inside rows of pitch
    size_t in_rows = 0, in_width = 0, in_pitch = 0;
    size_t out_rows = 0, out_width = 0, out_pitch = 0;
};

namespace {

void destroy_2d(mufft_plan_2d *pl)
{
    if (!pl)
        return;
    if (pl->device >= 0) {
        DeviceGuard g(pl->device);
        pl->res.release();
        pl->stage.release();
        if (pl->stream)
            cudaStreamDestroy(pl->stream);
    }
    delete pl;
}

mufft_plan_2d *create_2d(int kind, unsigned Nx, unsigned Ny, int direction, unsigned flags)
{
    t_err = 0;
    if (!is_pow2(Nx) || !is_pow2(Ny) || Nx == 1 || Ny == 1) {
        set_error(MUFFT_GB_ERR_INVALID, "Nx=%u, Ny=%u must be powers of two >= 2", Nx, Ny);
        return nullptr;
    }
    if (kind == K2_C2C && direction != MUFFT_FORWARD && direction != MUFFT_INVERSE) {
        set_error(MUFFT_GB_ERR_INVALID, "direction must be MUFFT_FORWARD or MUFFT_INVERSE");
        return nullptr;
    }
    if (kind != K2_C2C && Nx < 4) {
        set_error(MUFFT_GB_ERR_INVALID, "real 2D transforms need Nx >= 4");
        return nullptr;
    }
    const unsigned Mx = kind == K2_C2C ? Nx : Nx / 2;
    if (Mx > kMaxSinglePass || Ny > kMaxSinglePass) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "2D side longer than %u", kMaxSinglePass);
        return nullptr;
    }
    const TileKernel *krow = find_tile((int)Mx, ALONG, ALONG);
    const TileKernel *kcol = find_tile((int)Ny, ACROSS, ACROSS);
    if (!krow || !kcol) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "no 2D kernels for %u x %u", Nx, Ny);
        return nullptr;
    }
    int dev;
    if (!device_prepare(&dev))
        return nullptr;
    mufft_plan_2d *pl = new mufft_plan_2d();
    pl->device = dev;
    pl->kind = kind;
    pl->Nx = Nx;
    pl->Ny = Ny;
    pl->Mx = Mx;
    pl->flags = flags;
    pl->direction = kind == K2_C2C ? direction : (kind == K2_R2C ? MUFFT_FORWARD : MUFFT_INVERSE);
    const float2 *tw = g_dev[dev].tw;
    const bool inv = pl->direction == MUFFT_INVERSE;
    const bool full = (flags & MUFFT_FLAG_FULL_R2C) != 0;
    if (!cuda_ok(cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking), "cudaStreamCreate")) {
        destroy_2d(pl);
        return nullptr;
    }
    if (kind != K2_C2C) {
        pl->res.rtw = upload(r2c_twiddles(kind == K2_R2C ? MUFFT_FORWARD : MUFFT_INVERSE, Mx));
        if (!pl->res.rtw) {
            destroy_2d(pl);
            return nullptr;
        }
    }

    Pass row;
    row.k = krow;
    row.a.in_stride = 1;
    row.a.out_stride = 1;
    row.a.ntrans = Ny;
    row.a.tw = tw;
    row.a.rtw = pl->res.rtw;
    row.a.mirror_len = Mx;
    row.a.scale = 1.0f;
    row.grid = dim3((Ny + krow->C - 1) / krow->C, 1);

    Pass col;
    col.k = kcol;
    col.a.in_dist = 1;
    col.a.out_dist = 1;
    col.a.tw = tw;
    col.a.scale = 1.0f;

    if (kind == K2_C2C) {
        // rows then columns in place (fft.c:917-988)
        row.a.in_dist = Nx;
        row.a.out_dist = Nx;
        row.a.conj = inv ? 1 : 0;
        col.a.in_stride = col.a.out_stride = Nx;
        col.a.ntrans = Nx;
        col.a.conj = inv ? 2 : 0;
        col.in_role = ROLE_OUT;
        col.out_role = ROLE_OUT;
        pl->vertical_nx = Nx;
        pl->in_rows = pl->out_rows = Ny;
        pl->in_width = pl->out_width = pl->in_pitch = pl->out_pitch = (size_t)Nx * 8;
    } else if (kind == K2_R2C) {
        // rows with fused fix-up into a row stride of Nx complex, then the
        // Nx/2 + 1 (or Nx) columns in place (fft.c:939-987, :738-746)
        pl->vertical_nx = full ? Nx : Mx + 1;
        row.a.in_dist = Mx;
        row.a.out_dist = Nx;
        row.a.epilogue = full ? EPI_R2C_FULL : EPI_R2C;
        col.a.in_stride = col.a.out_stride = Nx;
        col.a.ntrans = pl->vertical_nx;
        col.in_role = ROLE_OUT;
        col.out_role = ROLE_OUT;
        pl->in_rows = Ny;
        pl->in_width = pl->in_pitch = (size_t)Nx * 4;
        pl->out_rows = Ny;
        pl->out_width = (size_t)pl->vertical_nx * 8;
        pl->out_pitch = (size_t)Nx * 8;
    } else {
        // columns first into scratch (Nx/2 + 1 of them), then rows with the
        // fused c2r fix-up (fft.c:863-916)
        pl->vertical_nx = Mx + 1;
        // rows of the Mx + 1 columns at a pitch of whole 128-byte lines: the
        // column tiles then store full sectors
        const size_t sstride = ((size_t)Mx + 1 + 15) & ~(size_t)15;
        pl->res.scratch_bytes = sstride * Ny * sizeof(float2);
        if (!cuda_ok(cudaMalloc(&pl->res.scratch, pl->res.scratch_bytes), "cudaMalloc(scratch)")) {
            destroy_2d(pl);
            return nullptr;
        }
        col.a.in_stride = Nx;
        col.a.out_stride = (long long)sstride;
        col.a.ntrans = Mx + 1;
        col.a.conj = 3;
        col.in_role = ROLE_IN;
        col.out_role = ROLE_SCRATCH;
        row.a.in_dist = (long long)sstride;
        row.a.out_dist = Mx;
        row.a.prologue = PRO_C2R;
        row.a.conj = 3;
        row.in_role = ROLE_SCRATCH;
        row.out_role = ROLE_OUT;
        pl->in_rows = Ny;
        pl->in_width = (size_t)(Mx + 1) * 8;
        pl->in_pitch = (size_t)Nx * 8;
        pl->out_rows = Ny;
        pl->out_width = pl->out_pitch = (size_t)Nx * 4;
    }
    col.grid = dim3((col.a.ntrans + kcol->C - 1) / kcol->C, 1);

    // Long columns: a four-step along the columns, Ny = N1 x N2, in two
    // passes of short column tiles (C1: length N1 at stride N2 rows, twiddle
    // W_Ny^(k1*n2) with n2 the grid row; C2: length N2, stored transposed to
    // rows k1 + N1*k2) -- 64-column tiles instead of the 1-2-column tiles a
    // whole 8192- or 16384-point column allows.  At Ny = 4096 the one-pass
    // 4-column tiles measured as fast or faster (4096^2 r2c columns 41.3 us
    // vs 18.6 + 26.8 us; c2c 84.8 vs 53.4 + 43.2 us), so the automatic choice
    // starts at 8192.
    const int mode = g_2d_columns.load();
    const unsigned lgy = ilog2u(Ny);
    const unsigned N1 = 1u << (lgy / 2), N2 = Ny / N1;
    const TileKernel *kc1 = find_tile((int)N1, ACROSS, ACROSS), *kc2 = find_tile((int)N2, ACROSS, ACROSS);
    if ((mode == 2 || (mode == 0 && Ny >= 8192)) && N1 >= 2 && kc1 && kc2) {
        const unsigned ncols = (unsigned)col.a.ntrans;
        const long long s_in = col.a.in_stride;                                 // pitch the columns are read at
        const long long s_out = kind == K2_C2R ? col.a.out_stride : (long long)Nx;  // pitch of C1 / C2 outputs
        const Role c1_in = kind == K2_C2R ? ROLE_IN : ROLE_SCRATCH;
        const Role c1_out = ROLE_SCRATCH;
        const Role c2_out = kind == K2_C2R ? ROLE_SCRATCH2 : ROLE_OUT;
        const size_t bytes = (size_t)Ny * (size_t)s_out * sizeof(float2);
        if (kind != K2_C2R) {
            cudaFree(pl->res.scratch);
            pl->res.scratch = nullptr;
        }
        if ((!pl->res.scratch && !cuda_ok(cudaMalloc(&pl->res.scratch, bytes), "cudaMalloc(scratch)")) ||
            (kind == K2_C2R && !cuda_ok(cudaMalloc(&pl->res.scratch2, bytes), "cudaMalloc(scratch)"))) {
            destroy_2d(pl);
            return nullptr;
        }
        Pass c1;
        c1.k = kc1;
        c1.a.tw = tw;
        c1.a.scale = 1.0f;
        c1.a.in_stride = (long long)N2 * s_in;
        c1.a.out_stride = (long long)N2 * s_out;
        c1.a.in_dist = c1.a.out_dist = 1;
        c1.a.in_batch = s_in;
        c1.a.out_batch = s_out;
        c1.a.ntrans = ncols;
        c1.a.conj = (col.a.conj & 1);
        c1.a.epilogue = EPI_TWIDDLE;
        c1.a.tw_by_y = 1;
        c1.a.tw_scale = 2.0f / (float)Ny;
        c1.a.tw_mask = Ny - 1;
        c1.in_role = c1_in;
        c1.out_role = c1_out;
        c1.grid = dim3((ncols + kc1->C - 1) / kc1->C, N2);
        Pass c2;
        c2.k = kc2;
        c2.a.tw = tw;
        c2.a.scale = 1.0f;
        c2.a.in_stride = s_out;
        c2.a.out_stride = (long long)N1 * s_out;
        c2.a.in_dist = c2.a.out_dist = 1;
        c2.a.in_batch = (long long)N2 * s_out;
        c2.a.out_batch = s_out;
        c2.a.ntrans = ncols;
        c2.a.conj = (col.a.conj & 2);
        c2.in_role = ROLE_SCRATCH;
        c2.out_role = c2_out;
        c2.grid = dim3((ncols + kc2->C - 1) / kc2->C, N1);
        if (kind == K2_C2R) {
            row.in_role = ROLE_SCRATCH2;
            pl->passes.push_back(c1);
            pl->passes.push_back(c2);
            pl->passes.push_back(row);
        } else {
            row.out_role = ROLE_SCRATCH;
            pl->passes.push_back(row);
            pl->passes.push_back(c1);
            pl->passes.push_back(c2);
        }
    } else if (kind == K2_C2R) {
        pl->passes.push_back(col);
        pl->passes.push_back(row);
    } else {
        pl->passes.push_back(row);
        pl->passes.push_back(col);
    }
    if (!attach_stream(pl->passes, false, pl->device) || !attach_occupancy(pl->passes, false, pl->device)) {
        destroy_2d(pl);
        return nullptr;
    }
    return pl;
}

int exec_2d(mufft_plan_2d *pl, void *out, const void *in, cudaStream_t st, bool sync)
{
    if (!pl || !out || !in) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan or buffer");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(pl->device);
    const bool hin = !is_device_accessible(in);
    const bool hout = !is_device_accessible(out);
    if (!sync && (hin || hout)) {
        set_error(MUFFT_GB_ERR_HOST_POINTER, "asynchronous execute needs device-accessible buffers");
        return MUFFT_GB_ERR_HOST_POINTER;
    }
    if (sync)
        st = pl->stream;
    Buffers b{in, out, nullptr, pl->res.scratch, pl->res.scratch2};
    const size_t in_bytes = pl->in_rows * pl->in_pitch;
    const size_t out_bytes = pl->out_rows * pl->out_pitch;
    if (hin) {
        if (!ensure(pl->stage.in, pl->stage.in_bytes, in_bytes))
            return t_err;
        if (!cuda_ok(cudaMemcpy2DAsync(pl->stage.in, pl->in_pitch, in, pl->in_pitch, pl->in_width,
                                       pl->in_rows, cudaMemcpyDefault, st),
                     "H2D copy"))
            return t_err;
        b.in = pl->stage.in;
    }
    if (hout) {
        if (!ensure(pl->stage.out, pl->stage.out_bytes, out_bytes))
            return t_err;
        b.out = pl->stage.out;
    }
    if (!cuda_ok(run_passes(pl->passes, b, st), "kernel launch"))
        return t_err;
    if (hout && !cuda_ok(cudaMemcpy2DAsync(out, pl->out_pitch, b.out, pl->out_pitch, pl->out_width,
                                           pl->out_rows, cudaMemcpyDefault, st),
                         "D2H copy"))
        return t_err;
    if (sync && !cuda_ok(cudaStreamSynchronize(st), "execute"))
        return t_err;
    return MUFFT_GB_OK;
}

}  // namespace

extern "C" {

mufft_plan_2d *mufft_create_plan_2d_c2c(unsigned Nx, unsigned Ny, int direction, unsigned flags)
{
    return create_2d(K2_C2C, Nx, Ny, direction, flags);
}

mufft_plan_2d *mufft_create_plan_2d_r2c(unsigned Nx, unsigned Ny, unsigned flags)
{
    return create_2d(K2_R2C, Nx, Ny, MUFFT_FORWARD, flags);
}

mufft_plan_2d *mufft_create_plan_2d_c2r(unsigned Nx, unsigned Ny, unsigned flags)
{
    return create_2d(K2_C2R, Nx, Ny, MUFFT_INVERSE, flags);
}

void mufft_execute_plan_2d(mufft_plan_2d *plan, void *MUFFT_RESTRICT output, const void *MUFFT_RESTRICT input)
{
    exec_2d(plan, output, input, nullptr, true);
}

int mufft_gb_execute_plan_2d_async(mufft_plan_2d *plan, void *output, const void *input, void *stream)
{
    return exec_2d(plan, output, input, (cudaStream_t)stream, false);
}

int mufft_gb_execute_plan_2d_launches_async(mufft_plan_2d *plan, void *output, const void *input, unsigned first,
                                            unsigned count, void *stream)
{
    if (!plan || !is_device_accessible(output) || !is_device_accessible(input)) {
        set_error(MUFFT_GB_ERR_INVALID, "needs a plan and device buffers");
        return MUFFT_GB_ERR_INVALID;
    }
    DeviceGuard g(plan->device);
    Buffers b{input, output, nullptr, plan->res.scratch, plan->res.scratch2};
    if (!cuda_ok(run_passes(plan->passes, b, (cudaStream_t)stream, first, count), "kernel launch"))
        return t_err;
    return MUFFT_GB_OK;
}

void mufft_free_plan_2d(mufft_plan_2d *plan) { destroy_2d(plan); }

unsigned mufft_gb_plan_2d_launches(const mufft_plan_2d *plan) { return plan ? (unsigned)plan->passes.size() : 0; }

int mufft_gb_plan_2d_describe(const mufft_plan_2d *plan, char *buf, size_t size)
{
    if (!plan || !buf || !size)
        return MUFFT_GB_ERR_INVALID;
    snprintf(buf, size, "%s", describe(plan->passes).c_str());
    return MUFFT_GB_OK;
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

// ========================================================= tile choice

int mufft_gb_set_twiddle_table(int mode)
{
    if (mode < -1 || mode > 2) {
        set_error(MUFFT_GB_ERR_INVALID, "mode must be -1 (automatic), 0, 1 or 2");
        return MUFFT_GB_ERR_INVALID;
    }
    g_twiddle_table.store(mode);
    return MUFFT_GB_OK;
}

int mufft_gb_autotune_1d(int kind, unsigned N, int direction, unsigned flags, unsigned batch, char *report,
                         size_t report_size)
{
    t_err = 0;
    if (kind < 0 || kind > 2) {
        set_error(MUFFT_GB_ERR_INVALID, "kind must be 0, 1 or 2");
        return MUFFT_GB_ERR_INVALID;
    }
    if (flags & (MUFFT_GB_FLAG_SPLIT_BF16X3 | MUFFT_GB_FLAG_SPLIT_BF16X2)) {
        set_error(MUFFT_GB_ERR_UNSUPPORTED, "split-precision plans have a single schedule");
        return MUFFT_GB_ERR_UNSUPPORTED;
    }
    flags &= ~MUFFT_GB_FLAG_AUTOTUNE;
    // validate the shape the way plan creation does (no device work)
    std::string dummy;
    create_1d(kind, N, direction, flags, batch, 0, 0, -1, true, &dummy);
    if (t_err)
        return t_err;
    int dev;
    if (!device_prepare(&dev))
        return t_err;
    PlanOptions best;
    std::string rep;
    if (!autotune_run(kind, N, direction, flags, batch, &best, &rep))
        return t_err ? t_err : MUFFT_GB_ERR_UNSUPPORTED;
    t_err = 0;
    if (report && report_size)
        snprintf(report, report_size, "%s", rep.c_str());
    return MUFFT_GB_OK;
}

void mufft_gb_autotune_clear(void)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.clear();
}

namespace {

bool device_identity(int *sms, std::string *name)
{
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        set_error(MUFFT_GB_ERR_NO_DEVICE, "no CUDA device visible");
        return false;
    }
    *sms = prop.multiProcessorCount;
    *name = prop.name;
    for (char &c : *name)
        if (c == ' ' || c == '\t' || c == '\n')
            c = '_';
    return true;
}

}  // namespace

// File format (text): a header line, the device line, then one line per shape:
//   entry <kind> <N> <batch> <flags> <levels> <twiddle> <fused> <ntiles> {<L> <lmap> <smap> <C> <R> <Q>}
int mufft_gb_autotune_save(const char *path)
{
    t_err = 0;
    int sms;
    std::string name;
    if (!path) {
        set_error(MUFFT_GB_ERR_INVALID, "null path");
        return MUFFT_GB_ERR_INVALID;
    }
    if (!device_identity(&sms, &name))
        return t_err;
    FILE *f = fopen(path, "w");
    if (!f) {
        set_error(MUFFT_GB_ERR_INVALID, "cannot write %s", path);
        return MUFFT_GB_ERR_INVALID;
    }
    fprintf(f, "mufft_gb300-autotune 2\ndevice %d %s\n", sms, name.c_str());
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        for (const auto &kv : g_tune) {
            const PlanOptions &o = kv.second;
            fprintf(f, "entry %d %u %u %u %d %d %d %d %zu", kv.first.kind, kv.first.N, kv.first.batch, kv.first.flags,
                    o.levels, o.twiddle, o.fused, o.tma, o.tiles.size());
            for (const TileKernel &k : o.tiles)
                fprintf(f, " %d %d %d %d %d %d", k.L, k.lmap, k.smap, k.C, k.R, k.Q);
            fprintf(f, "\n");
        }
    }
    const bool ok = fclose(f) == 0;
    if (!ok) {
        set_error(MUFFT_GB_ERR_INVALID, "cannot write %s", path);
        return MUFFT_GB_ERR_INVALID;
    }
    return MUFFT_GB_OK;
}

int mufft_gb_autotune_load(const char *path)
{
    t_err = 0;
    int sms;
    std::string name;
    if (!path) {
        set_error(MUFFT_GB_ERR_INVALID, "null path");
        return MUFFT_GB_ERR_INVALID;
    }
    FILE *f = fopen(path, "r");
    if (!f) {
        set_error(MUFFT_GB_ERR_INVALID, "cannot read %s", path);
        return MUFFT_GB_ERR_INVALID;
    }
    char line[4096], fname[256];
    int fsms = -1, version = 0;
    bool ok = fgets(line, sizeof(line), f) && sscanf(line, "mufft_gb300-autotune %d", &version) == 1 && version == 2 &&
              fgets(line, sizeof(line), f) && sscanf(line, "device %d %255s", &fsms, fname) == 2;
    if (!ok) {
        fclose(f);
        set_error(MUFFT_GB_ERR_INVALID, "%s is not an autotune cache", path);
        return MUFFT_GB_ERR_INVALID;
    }
    if (!device_identity(&sms, &name)) {
        fclose(f);
        return t_err;
    }
    if (fsms != sms || name != fname) {
        fclose(f);
        set_error(MUFFT_GB_ERR_INVALID, "autotune cache was made on another GPU (%s, %d SMs)", fname, fsms);
        return MUFFT_GB_ERR_INVALID;
    }
    std::map<TuneKey, PlanOptions> loaded;
    while (fgets(line, sizeof(line), f)) {
        TuneKey k{};
        PlanOptions o;
        size_t nt = 0;
        int used = 0;
        if (sscanf(line, "entry %d %u %u %u %d %d %d %d %zu%n", &k.kind, &k.N, &k.batch, &k.flags, &o.levels,
                   &o.twiddle, &o.fused, &o.tma, &nt, &used) != 9 || nt > 16)
            continue;
        const char *q = line + used;
        bool good = true;
        for (size_t i = 0; i < nt && good; i++) {
            int L, lm, sm, C, R, Q, n = 0;
            good = sscanf(q, "%d %d %d %d %d %d%n", &L, &lm, &sm, &C, &R, &Q, &n) == 6;
            q += n;
            const TileKernel *tk = good ? find_tile(L, lm, sm, C, R, Q) : nullptr;
            good = tk && tk->C == C && tk->R == R && tk->Q == Q;
            if (good)
                o.tiles.push_back(*tk);
        }
        if (good)
            loaded[k] = o;
    }
    fclose(f);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    for (const auto &kv : loaded)
        g_tune[kv.first] = kv.second;
    return MUFFT_GB_OK;
}

int mufft_gb_set_conv_classes(unsigned points)
{
    if (points != 0 && (!is_pow2(points) || points < (1u << kRaggedMinSplitLg) || points > 65536)) {
        set_error(MUFFT_GB_ERR_INVALID, "class size must be 0 or a power of two in 16384..65536");
        return MUFFT_GB_ERR_INVALID;
    }
    g_conv_class_lg.store(points ? ilog2u(points) : 17u);
    return MUFFT_GB_OK;
}

int mufft_gb_set_conv_split(unsigned points)
{
    if (points != 0 && (!is_pow2(points) || points < (1u << kRaggedMinSplitLg) || points > 65536)) {
        set_error(MUFFT_GB_ERR_INVALID, "split size must be 0 or a power of two in 16384..65536");
        return MUFFT_GB_ERR_INVALID;
    }
    g_conv_split_lg.store(points ? ilog2u(points) : 17u);
    return MUFFT_GB_OK;
}

int mufft_gb_set_2d_columns(int mode)
{
    if (mode < 0 || mode > 2) {
        set_error(MUFFT_GB_ERR_INVALID, "mode must be 0 (automatic), 1 (one pass) or 2 (two passes)");
        return MUFFT_GB_ERR_INVALID;
    }
    g_2d_columns.store(mode);
    return MUFFT_GB_OK;
}

int mufft_gb_set_tma(int mode)
{
    if (mode < 0 || mode > 2) {
        set_error(MUFFT_GB_ERR_INVALID, "mode must be 0 (off), 1 (double-buffered) or 2 (single buffer)");
        return MUFFT_GB_ERR_INVALID;
    }
    g_tma.store(mode);
    return MUFFT_GB_OK;
}

int mufft_gb_set_stream_tiles(int enable)
{
    if (enable < 0 || enable > 1) {
        set_error(MUFFT_GB_ERR_INVALID, "enable must be 0 or 1");
        return MUFFT_GB_ERR_INVALID;
    }
    g_stream.store(enable);
    return MUFFT_GB_OK;
}

int mufft_gb_set_tile_occupancy(int ctas_per_sm)
{
    if (ctas_per_sm < 0 || ctas_per_sm > 32) {
        set_error(MUFFT_GB_ERR_INVALID, "CTAs per SM must be 0 (no cap) .. 32");
        return MUFFT_GB_ERR_INVALID;
    }
    g_occ.store(ctas_per_sm);
    return MUFFT_GB_OK;
}

int mufft_gb_set_split_engine(int engine)
{
    if (engine < 0 || engine > 1) {
        set_error(MUFFT_GB_ERR_INVALID, "engine must be 0 (tcgen05) or 1 (mma.sync)");
        return MUFFT_GB_ERR_INVALID;
    }
    g_split_engine.store(engine);
    return MUFFT_GB_OK;
}

int mufft_gb_set_fused_passes(int enable)
{
    g_fused_bc.store(enable ? 1 : 0);
    return MUFFT_GB_OK;
}

int mufft_gb_set_multipass_levels(unsigned levels)
{
    if (levels != 0 && levels != 2 && levels != 3) {
        set_error(MUFFT_GB_ERR_INVALID, "levels must be 0 (automatic), 2 or 3");
        return MUFFT_GB_ERR_INVALID;
    }
    g_levels.store((int)levels);
    return MUFFT_GB_OK;
}

int mufft_gb_set_tile_choice(unsigned L, int load_across, int store_across, unsigned transforms_per_tile,
                             unsigned elems_per_thread, unsigned cluster_ctas)
{
    if (!set_tile_choice((int)L, load_across ? ACROSS : ALONG, store_across ? ACROSS : ALONG,
                         (int)transforms_per_tile, (int)elems_per_thread, (int)cluster_ctas)) {
        set_error(MUFFT_GB_ERR_INVALID, "no tile kernel L=%u C=%u R=%u Q=%u for that map", L, transforms_per_tile,
                  elems_per_thread, cluster_ctas);
        return MUFFT_GB_ERR_INVALID;
    }
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
