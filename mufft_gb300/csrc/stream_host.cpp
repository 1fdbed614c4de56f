// Streaming partitioned convolution, host side: filter partition spectra,
// the delay line, and one block per launch (stream_conv.cu) or per graph of
// launches (misc_kernels.cu's multiply-accumulate between two row tiles).
#include <algorithm>

#include "host.h"
#include "misc_kernels.h"
#include "stream_conv.h"

using namespace mgb;

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
                                                  unsigned flags, const mufft_gb_options *opts)
{
    t_err = 0;
    mufft_gb_options o;
    PlanOptions po;
    if (!public_options(opts, &o) || (opts && !convert_options(opts, &po)))
        return nullptr;
    OptionsScope scope(opts ? &po : nullptr);
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
    // The one-launch block needs both window transforms as one 256-thread
    // row tile of 4096 / M transforms (M complex points each): ask for that
    // tile unless the caller's options choose one.
    const unsigned M = stereo ? L : L / 2;
    PlanOptions wopts = opts ? po : PlanOptions();
    if (o.stream_conv_fused && upols_block_supported((int)M)) {
        bool chosen = false;
        for (const TileKernel &k : wopts.tiles)
            chosen = chosen || (k.L == (int)M && k.lmap == ALONG && k.smap == ALONG);
        const TileKernel *k = chosen ? nullptr : find_tile((int)M, ALONG, ALONG, 4096 / (int)M, 16, 1);
        if (k)
            wopts.tiles.push_back(*k);
    }
    {
        OptionsScope wscope(&wopts);
        c->fwd = create_1d(stereo ? K_C2C : K_R2C, L, MUFFT_FORWARD, tflags, 1, 0, 0, -1, false, nullptr);
        c->inv = create_1d(stereo ? K_C2C : K_C2R, L, MUFFT_INVERSE, tflags, 1, 0, 0, -1, false, nullptr);
    }
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
    const unsigned want_ranges = o.stream_conv_ranges;
    // One launch per block when both transforms are one 256-thread row tile
    auto row_tile = [M](const mufft_plan_1d *pl) {
        if (pl->passes.size() != 1)
            return false;
        const Pass &p = pl->passes[0];
        return p.type == PASS_TILE && p.k && !p.tk && !p.sk && p.smem_min == 0 && p.k->Q == 1 && p.k->R == 16 &&
               p.k->lmap == ALONG && p.k->smap == ALONG && p.k->L == (int)M && p.k->C * p.k->L == 4096 &&
               p.grid.x == 1 && p.grid.y == 1 && p.in_role == ROLE_IN && p.out_role == ROLE_OUT;
    };
    if (o.stream_conv_fused && upols_block_supported((int)M) && row_tile(c->fwd) && row_tile(c->inv)) {
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

unsigned mufft_gb_stream_conv_ranges(const mufft_gb_stream_conv *c) { return c ? c->G : 0u; }

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
