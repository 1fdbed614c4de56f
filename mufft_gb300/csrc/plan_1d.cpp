// 1D plans: the reference's mufft_create_plan_1d_* / mufft_execute_plan_1d
// (fft.c:476-547, 626-662, 811-850) with the same argument checks and NULL
// returns, batches, asynchronous execution, and the autotuner that measures
// the GPU schedule of a plan shape and remembers the fastest.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>

#include "host.h"

namespace mgb {

}  // namespace mgb

void mufft_plan_1d::Pipeline::release()
{
    for (int i = 0; i < 2; i++) {
        cudaFree(in[i]);
        cudaFree(out[i]);
        in[i] = out[i] = nullptr;
        for (cudaEvent_t *e : {&in_ready[i], &computed[i], &in_free[i], &out_free[i]})
            if (*e) {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
    }
    for (cudaStream_t &s : st)
        if (s) {
            cudaStreamDestroy(s);
            s = nullptr;
        }
    ready = false;
}

namespace mgb {

void destroy_1d(mufft_plan_1d *pl)
{
    if (!pl)
        return;
    if (pl->device >= 0) {
        DeviceGuard g(pl->device);
        pl->res.release();
        pl->stage.release();
        pl->pipe.release();
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
static std::mutex g_tune_mu;
static std::map<TuneKey, PlanOptions> g_tune;

static bool tune_lookup(int kind, unsigned N, unsigned batch, unsigned flags, PlanOptions *o)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(TuneKey{kind, N, batch, flags & kTuneFlagMask});
    if (it == g_tune.end())
        return false;
    *o = it->second;
    return true;
}

static bool autotune_run(int kind, unsigned N, int direction, unsigned flags, unsigned batch, PlanOptions *best,
                         std::string *report);

mufft_plan_1d *create_1d(int kind, unsigned N, int direction, unsigned flags, unsigned batch,
                         size_t idist, size_t odist, int prologue_override, bool dry,
                         std::string *desc, bool conj2)
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
        p.sp_engine = opt_split_engine();
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
                           attach_persist(pl->passes, dry, pl->device) &&
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

static std::string describe_options(const PlanOptions &o)
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
static bool autotune_run(int kind, unsigned N, int direction, unsigned flags, unsigned batch, PlanOptions *best,
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

}  // namespace mgb

using namespace mgb;

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

mufft_plan_1d *mufft_gb_create_plan_1d(int kind, unsigned N, int direction, unsigned flags, unsigned batch,
                                       size_t idist, size_t odist, const mufft_gb_options *opts)
{
    t_err = 0;
    if (kind < 0 || kind > 2) {
        set_error(MUFFT_GB_ERR_INVALID, "kind must be 0 (c2c), 1 (r2c) or 2 (c2r)");
        return nullptr;
    }
    PlanOptions o;
    if (opts && !convert_options(opts, &o))
        return nullptr;
    OptionsScope scope(opts ? &o : nullptr);
    return create_1d(kind, N, kind == K_C2C ? direction : (kind == K_R2C ? MUFFT_FORWARD : MUFFT_INVERSE), flags,
                     batch, idist, odist, -1, false, nullptr);
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

// Transforms `count` inputs into `count` outputs with the copies of one
// transform overlapping the kernels and copies of its neighbours: input i + 1
// is copied in while transform i runs and output i - 1 is copied out.
int mufft_gb_execute_plan_1d_host_pipeline(mufft_plan_1d *plan, void *const *outputs, const void *const *inputs,
                                           unsigned count)
{
    if (!plan || (count && (!outputs || !inputs))) {
        set_error(MUFFT_GB_ERR_INVALID, "null plan or buffer lists");
        return MUFFT_GB_ERR_INVALID;
    }
    if (plan->uses_in2) {
        set_error(MUFFT_GB_ERR_INVALID, "plan needs two inputs");
        return MUFFT_GB_ERR_INVALID;
    }
    for (unsigned i = 0; i < count; i++)
        if (!outputs[i] || !inputs[i]) {
            set_error(MUFFT_GB_ERR_INVALID, "null buffer %u", i);
            return MUFFT_GB_ERR_INVALID;
        }
    t_err = 0;
    DeviceGuard g(plan->device);
    mufft_plan_1d::Pipeline &P = plan->pipe;
    const size_t ib = plan->in_total(), ob = plan->out_total();
    if (!P.ready) {
        bool ok = true;
        for (int i = 0; i < 2 && ok; i++)
            ok = cuda_ok(cudaMalloc(&P.in[i], ib), "cudaMalloc(pipeline)") &&
                 cuda_ok(cudaMalloc(&P.out[i], ob), "cudaMalloc(pipeline)") &&
                 cuda_ok(cudaEventCreateWithFlags(&P.in_ready[i], cudaEventDisableTiming), "cudaEventCreate") &&
                 cuda_ok(cudaEventCreateWithFlags(&P.computed[i], cudaEventDisableTiming), "cudaEventCreate") &&
                 cuda_ok(cudaEventCreateWithFlags(&P.in_free[i], cudaEventDisableTiming), "cudaEventCreate") &&
                 cuda_ok(cudaEventCreateWithFlags(&P.out_free[i], cudaEventDisableTiming), "cudaEventCreate");
        for (int s = 0; s < 3 && ok; s++)
            ok = cuda_ok(cudaStreamCreateWithFlags(&P.st[s], cudaStreamNonBlocking), "cudaStreamCreate");
        if (!ok) {
            P.release();
            return t_err;
        }
        P.ready = true;
    }
    cudaStream_t cin = P.st[0], comp = P.st[1], cout = P.st[2];
    for (unsigned i = 0; i < count; i++) {
        const int s = (int)(i & 1);
        // input slot s is free once transform i - 2 has read it; output slot s
        // once output i - 2 has been copied out
        if (i >= 2 && !cuda_ok(cudaStreamWaitEvent(cin, P.in_free[s], 0), "pipeline"))
            return t_err;
        if (!cuda_ok(cudaMemcpyAsync(P.in[s], inputs[i], ib, cudaMemcpyDefault, cin), "H2D copy") ||
            !cuda_ok(cudaEventRecord(P.in_ready[s], cin), "pipeline") ||
            !cuda_ok(cudaStreamWaitEvent(comp, P.in_ready[s], 0), "pipeline") ||
            (i >= 2 && !cuda_ok(cudaStreamWaitEvent(comp, P.out_free[s], 0), "pipeline")))
            return t_err;
        Buffers b{P.in[s], P.out[s], nullptr, plan->res.scratch};
        if (!cuda_ok(run_passes(plan->passes, b, comp), "kernel launch") ||
            !cuda_ok(cudaEventRecord(P.in_free[s], comp), "pipeline") ||
            !cuda_ok(cudaEventRecord(P.computed[s], comp), "pipeline") ||
            !cuda_ok(cudaStreamWaitEvent(cout, P.computed[s], 0), "pipeline") ||
            !cuda_ok(cudaMemcpyAsync(outputs[i], P.out[s], ob, cudaMemcpyDefault, cout), "D2H copy") ||
            !cuda_ok(cudaEventRecord(P.out_free[s], cout), "pipeline"))
            return t_err;
    }
    for (cudaStream_t st : {cin, comp, cout})
        if (!cuda_ok(cudaStreamSynchronize(st), "execute"))
            return t_err;
    if (plan->res.err) {
        int e = 0;
        if (cuda_ok(cudaMemcpy(&e, plan->res.err, sizeof(int), cudaMemcpyDeviceToHost), "error flag") && e) {
            set_error(MUFFT_GB_ERR_UNSUPPORTED, "a bounded wait in a persistent kernel timed out");
            cudaMemset(plan->res.err, 0, sizeof(int));
            return t_err;
        }
    }
    return MUFFT_GB_OK;
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
                                  const mufft_gb_options *opts, char *buf, size_t size)
{
    std::string d;
    if (kind < 0 || kind > 2) {
        set_error(MUFFT_GB_ERR_INVALID, "kind must be 0, 1 or 2");
        return MUFFT_GB_ERR_INVALID;
    }
    t_err = 0;
    PlanOptions o;
    if (opts && !convert_options(opts, &o))
        return t_err;
    OptionsScope scope(opts ? &o : nullptr);
    create_1d(kind, N, direction, flags, batch, 0, 0, -1, true, &d);
    if (t_err)
        return t_err;
    if (buf && size)
        snprintf(buf, size, "%s", d.c_str());
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

}  // extern "C"

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

extern "C" {

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

}  // extern "C"
