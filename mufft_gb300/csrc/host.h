// Host-side internals shared by the translation units of the C API:
// errors, device state, per-plan options, the launch schedule ("passes") and
// the 1D plan that every other plan kind is built from.
//
//   host_common.cpp   errors, kernel registry lookups, options, device state,
//                     FP64 tables, memory helpers
//   schedule.cpp      passes: launch, describe, build (single pass, four-step,
//                     three-level), TMA / streaming / occupancy variants
//   plan_1d.cpp       mufft_plan_1d (fft.h 1D API, batches, async) and the
//                     autotuner with its cache
//   plan_2d.cpp       mufft_plan_2d
//   conv.cpp          mufft_plan_conv, mufft_get_convolve_func, the batched
//                     convolution output and the adjoints
//   conv_batch.cpp    ragged batched convolution (host side of conv_ragged.cu)
//   fft_batch.cpp     ragged batched transforms (host side of fft_ragged.cu)
//   stream_host.cpp   streaming partitioned convolution (host side of
//                     stream_conv.cu)
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/fft.h"
#include "../../include/mufft_gb300.h"
#include "bc_fused.h"
#include "common.h"
#include "registry.h"
#include "split_tc.h"
#include "tiles_persist.h"
#include "tiles_stream.h"
#include "tiles_tma.h"

namespace mgb {

// ------------------------------------------------------------------ errors

// Last error of the calling thread (mufft_gb_last_error) and its text.
extern thread_local int t_err;
extern thread_local char t_errmsg[512];
void set_error(int code, const char *fmt, ...);
bool cuda_ok(cudaError_t e, const char *what);

inline bool is_pow2(unsigned n) { return n != 0 && (n & (n - 1)) == 0; }
inline unsigned ilog2u(unsigned long long n)
{
    unsigned l = 0;
    while ((1ull << l) < n)
        l++;
    return l;
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev);
    ~DeviceGuard();
};

// ---------------------------------------------------------------- registry

const std::vector<TileKernel> &tile_table();
const TmaTileKernel *find_tma(int L, int R, int C, int nbuf);
const StreamTileKernel *find_stream(int L, int R, int C);
const PersistTileKernel *find_persist(int L, int R, int C, int lmap, int smap);

// ----------------------------------------------------------------- options

// Schedule choices of one plan: the public mufft_gb_options, or a candidate
// of the autotuner, or its remembered choice for a shape.  -2 leaves a
// field at its built-in default; `tiles` are preferred (L, lmap, smap) ->
// (C, R, Q).
struct PlanOptions {
    int levels = -2, twiddle = -2, fused = -2, tma = -2, occ = -2, stream = -2, split_engine = -2, cols2d = -2,
        persist = -2, l2 = -2;
    std::vector<TileKernel> tiles;
};
// The options of the plan being built on this thread (null: defaults).
extern thread_local const PlanOptions *t_opts;

// Sets t_opts for the lifetime of the guard (and restores the previous value).
struct OptionsScope {
    const PlanOptions *prev;
    explicit OptionsScope(const PlanOptions *o) : prev(t_opts) { t_opts = o; }
    ~OptionsScope() { t_opts = prev; }
};

// Validates public options and converts them (all fields explicit).
bool convert_options(const mufft_gb_options *in, PlanOptions *out);
// The public options with defaults where `in` is null (validated).
bool public_options(const mufft_gb_options *in, mufft_gb_options *out);

int opt_levels();
int opt_twiddle();
int opt_fused();
int opt_tma();
int opt_occ();
int opt_stream();
int opt_split_engine();
int opt_cols2d();
int opt_persist();
int opt_l2();

// ------------------------------------------------------------ device state

struct DeviceState {
    bool ready = false;
    float2 *tw = nullptr;  // stage twiddle table (common.h: stage_table_base)
};
constexpr int kMaxDevices = 64;
extern DeviceState g_dev[kMaxDevices];
// Makes sure the current device has its twiddle table and kernel attributes.
bool device_prepare(int *dev_out);

// i*dir*exp(i*pi*dir*k/M) for k < M, FP64 then rounded (fft.c:441-455).
std::vector<float2> r2c_twiddles(int dir, unsigned M);
float2 *upload(const std::vector<float2> &h);
bool is_device_accessible(const void *p);

// ------------------------------------------------------------------ passes

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
    // the tiles as a persistent grid (tiles_persist.cu); `k` is the same tile
    // as one launch per tile
    const PersistTileKernel *pt = nullptr;
    unsigned pt_grid = 0;
};

struct Buffers {
    const void *in;
    void *out;
    const void *in2;
    void *scratch;
    void *scratch2 = nullptr;
};

cudaError_t run_passes(const std::vector<Pass> &ps, const Buffers &b, cudaStream_t st, size_t first = 0,
                       size_t count = (size_t)-1);
std::string describe(const std::vector<Pass> &ps);

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
    void release();
};

bool build_fft_passes(const FftSpec &s, const float2 *tw, PlanResources &res, bool dry, std::vector<Pass> &out);
bool attach_tma(std::vector<Pass> &ps, PlanResources &res, bool dry, int device);
bool attach_stream(std::vector<Pass> &ps, bool dry, int device);
bool attach_persist(std::vector<Pass> &ps, bool dry, int device);
bool attach_occupancy(std::vector<Pass> &ps, bool dry, int device);

// Lazily allocated device staging for host-memory arguments.
struct Staging {
    void *in = nullptr, *out = nullptr, *in2 = nullptr;
    size_t in_bytes = 0, out_bytes = 0, in2_bytes = 0;
    void release();
};
bool ensure(void *&p, size_t &have, size_t need);

// ------------------------------------------------------------------ 1D plan

enum Kind1D { K_C2C = 0, K_R2C = 1, K_C2R = 2 };

}  // namespace mgb

struct mufft_plan_1d {
    int device = -1;
    int kind = mgb::K_C2C;
    unsigned N = 0, M = 0;
    int direction = MUFFT_FORWARD;
    unsigned flags = 0;
    unsigned batch = 1;
    size_t in_elem = 8, out_elem = 8;    // bytes per input / output element
    size_t in_count = 0, out_count = 0;  // elements read / written per transform
    size_t idist = 0, odist = 0;         // elements between transforms
    std::vector<mgb::Pass> passes;
    mgb::PlanResources res;
    mgb::Staging stage;
    cudaStream_t stream = nullptr;
    bool uses_in2 = false;
    // pipelined host execution (mufft_gb_execute_plan_1d_host_pipeline): two
    // device input and output slots, a copy-in, a compute and a copy-out
    // stream, made on first use
    struct Pipeline {
        void *in[2] = {nullptr, nullptr}, *out[2] = {nullptr, nullptr};
        cudaStream_t st[3] = {nullptr, nullptr, nullptr};
        cudaEvent_t in_ready[2] = {}, computed[2] = {}, in_free[2] = {}, out_free[2] = {};
        bool ready = false;
        void release();
    } pipe;

    size_t in_total() const { return ((size_t)(batch - 1) * idist + in_count) * in_elem; }
    size_t out_total() const { return ((size_t)(batch - 1) * odist + out_count) * out_elem; }
};

namespace mgb {

void destroy_1d(mufft_plan_1d *pl);
// prologue_override: PRO_MUL / PRO_MUL_C2R for convolution output plans
// (conj2: multiply by the conjugate, the adjoint).  Uses t_opts, or the
// autotuner's remembered choice for the shape when t_opts is null.
mufft_plan_1d *create_1d(int kind, unsigned N, int direction, unsigned flags, unsigned batch, size_t idist,
                         size_t odist, int prologue_override, bool dry, std::string *desc, bool conj2 = false);
// Runs a 1D plan; `sync` selects the fft.h semantics (any memory, blocking).
int exec_1d(mufft_plan_1d *pl, void *out, const void *in, const void *in2, cudaStream_t st, bool sync);

}  // namespace mgb
