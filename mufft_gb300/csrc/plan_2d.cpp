// 2D plans: the reference's mufft_create_plan_2d_* / mufft_execute_plan_2d
// (fft.c:664-792, 852-989) -- row transforms, the r2c / c2r fix-up fused
// into the row pass, column transforms across rows.
#include <cstdio>

#include "host.h"

using namespace mgb;

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

// dry: the schedule only (into `desc`), without touching a GPU; returns null.
mufft_plan_2d *create_2d(int kind, unsigned Nx, unsigned Ny, int direction, unsigned flags, bool dry = false,
                         std::string *desc = nullptr)
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
    int dev = 0;
    if (!dry && !device_prepare(&dev))
        return nullptr;
    mufft_plan_2d *pl = new mufft_plan_2d();
    pl->device = dev;
    pl->kind = kind;
    pl->Nx = Nx;
    pl->Ny = Ny;
    pl->Mx = Mx;
    pl->flags = flags;
    pl->direction = kind == K2_C2C ? direction : (kind == K2_R2C ? MUFFT_FORWARD : MUFFT_INVERSE);
    const float2 *tw = dry ? nullptr : g_dev[dev].tw;
    const bool inv = pl->direction == MUFFT_INVERSE;
    const bool full = (flags & MUFFT_FLAG_FULL_R2C) != 0;
    if (!dry && !cuda_ok(cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking), "cudaStreamCreate")) {
        destroy_2d(pl);
        return nullptr;
    }
    if (kind != K2_C2C && !dry) {
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
        if (!dry && !cuda_ok(cudaMalloc(&pl->res.scratch, pl->res.scratch_bytes), "cudaMalloc(scratch)")) {
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
    // whole 8192- or 16384-point column allows.  With the intermediate kept in
    // L2 (cache-policy hints) the two passes also win at Ny = 4096 for wide
    // grids; measured (us, r2c / c2r / c2c, one pass -> two passes): 4096 x
    // 4096 72.0 / 82.7 / 125.9 -> 69.1 / 79.5 / 130.1, 8192 x 4096 160.1 /
    // 160.4 / 313.7 -> 141.5 / 159.5 / 289.0, 16384 x 4096 356.2 / 397.2 /
    // 708.9 -> 306.9 / 358.9 / 633.3, but 2048 x 4096 39.1 / 43.9 / 65.8 ->
    // 41.1 / 44.7 / 63.0 and 4096 x 2048 or 16384 x 2048 slower in every
    // kind.  So the automatic choice: Ny >= 8192, or Ny = 4096 with Nx >= 4096
    // (real) / Nx >= 8192 (c2c); without the hints one pass up to 4096.
    const int mode = opt_cols2d();
    const unsigned lgy = ilog2u(Ny);
    const unsigned N1 = 1u << (lgy / 2), N2 = Ny / N1;
    const TileKernel *kc1 = find_tile((int)N1, ACROSS, ACROSS), *kc2 = find_tile((int)N2, ACROSS, ACROSS);
    const bool wide = opt_l2() == 1 && Ny >= 4096 && Nx >= (kind == K2_C2C ? 8192u : 4096u);
    if ((mode == 2 || (mode == 0 && (Ny >= 8192 || wide))) && N1 >= 2 && kc1 && kc2) {
        const unsigned ncols = (unsigned)col.a.ntrans;
        const long long s_in = col.a.in_stride;                                 // pitch the columns are read at
        const long long s_out = kind == K2_C2R ? col.a.out_stride : (long long)Nx;  // pitch of C1 / C2 outputs
        const Role c1_in = kind == K2_C2R ? ROLE_IN : ROLE_SCRATCH;
        const Role c1_out = ROLE_SCRATCH;
        const Role c2_out = kind == K2_C2R ? ROLE_SCRATCH2 : ROLE_OUT;
        const size_t bytes = (size_t)Ny * (size_t)s_out * sizeof(float2);
        if (kind != K2_C2R && !dry) {
            cudaFree(pl->res.scratch);
            pl->res.scratch = nullptr;
        }
        if (!dry && ((!pl->res.scratch && !cuda_ok(cudaMalloc(&pl->res.scratch, bytes), "cudaMalloc(scratch)")) ||
                     (kind == K2_C2R && !cuda_ok(cudaMalloc(&pl->res.scratch2, bytes), "cudaMalloc(scratch)")))) {
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
        if (opt_l2() == 1) {
            // intermediates kept in L2 and dropped once read, as in the
            // one-pass forms: C2 reads whole 128-byte lines of C1's output
            // (64-column tiles at a pitch of whole lines) when its tile is at
            // least 16 columns wide
            const bool lines = kc2->C >= 16 && (s_out % 16) == 0;
            c1.a.l2 = kind == K2_C2R ? (L2_LOAD_FIRST | L2_STORE_LAST) : L2_STORE_LAST;
            c2.a.l2 = (lines ? L2_DISCARD_IN : 0) | (kind == K2_C2R ? L2_STORE_LAST : L2_STORE_FIRST);
            if (kind == K2_C2R)
                row.a.l2 = L2_DISCARD_IN | L2_STORE_FIRST;
            else
                row.a.l2 = L2_LOAD_FIRST | L2_STORE_LAST;
        }
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
        if (opt_l2() == 1) {
            // the column pass's output is the row pass's input only: kept in
            // L2, dropped without write-back once read (rows of the scratch
            // are whole 128-byte lines apart)
            col.a.l2 = L2_LOAD_FIRST | L2_STORE_LAST;
            row.a.l2 = L2_DISCARD_IN | L2_STORE_FIRST;
        }
        pl->passes.push_back(col);
        pl->passes.push_back(row);
    } else {
        if (opt_l2() == 1)  // the rows' output is what the column pass reads next
            row.a.l2 = L2_LOAD_FIRST | L2_STORE_LAST;
        pl->passes.push_back(row);
        pl->passes.push_back(col);
    }
    if (!attach_stream(pl->passes, dry, pl->device) || !attach_persist(pl->passes, dry, pl->device) ||
        !attach_occupancy(pl->passes, dry, pl->device)) {
        if (dry)
            delete pl;
        else
            destroy_2d(pl);
        return nullptr;
    }
    if (desc)
        *desc = describe(pl->passes);
    if (dry) {
        delete pl;  // nothing was allocated
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

mufft_plan_2d *mufft_gb_create_plan_2d(int kind, unsigned Nx, unsigned Ny, int direction, unsigned flags,
                                       const mufft_gb_options *opts)
{
    t_err = 0;
    if (kind < K2_C2C || kind > K2_C2R) {
        set_error(MUFFT_GB_ERR_INVALID, "kind must be 0 (c2c), 1 (r2c) or 2 (c2r)");
        return nullptr;
    }
    PlanOptions o;
    if (opts && !convert_options(opts, &o))
        return nullptr;
    OptionsScope scope(opts ? &o : nullptr);
    return create_2d(kind, Nx, Ny, kind == K2_C2C ? direction : (kind == K2_R2C ? MUFFT_FORWARD : MUFFT_INVERSE),
                     flags);
}

int mufft_gb_describe_schedule_2d(int kind, unsigned Nx, unsigned Ny, int direction, unsigned flags,
                                  const mufft_gb_options *opts, char *buf, size_t size)
{
    t_err = 0;
    if (kind < K2_C2C || kind > K2_C2R) {
        set_error(MUFFT_GB_ERR_INVALID, "kind must be 0 (c2c), 1 (r2c) or 2 (c2r)");
        return MUFFT_GB_ERR_INVALID;
    }
    PlanOptions o;
    if (opts && !convert_options(opts, &o))
        return t_err;
    OptionsScope scope(opts ? &o : nullptr);
    std::string d;
    create_2d(kind, Nx, Ny, kind == K2_C2C ? direction : (kind == K2_R2C ? MUFFT_FORWARD : MUFFT_INVERSE), flags,
              true, &d);
    if (t_err)
        return t_err;
    if (buf && size)
        snprintf(buf, size, "%s", d.c_str());
    return MUFFT_GB_OK;
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

}  // extern "C"
