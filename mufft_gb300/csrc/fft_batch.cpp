// Ragged batched transforms, host side: request checks, the task order of
// the persistent kernel (fft_ragged.cu) and the CUDA graph that replays a
// batch.  The per-request equivalent is one reference plan per request
// (mufft_create_plan_1d_c2c / _r2c / _c2r, fft.c:476-547, 626-662) and one
// mufft_execute_plan_1d each (fft.c:811-850).
#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>

#include "fft_ragged.h"
#include "host.h"

using namespace mgb;

struct mufft_gb_fft_batch {
    int device = -1;
    unsigned count = 0;
    std::vector<FftRaggedReq> sorted;  // longest first (host copy, scratch assigned)
    FftRaggedReq *d_reqs = nullptr;
    FftRaggedTask *d_tasks = nullptr;
    const float2 **d_tab = nullptr;
    unsigned *d_next = nullptr;        // [0] dequeue counter, [1 + c] split request c
    size_t next_bytes = 0;
    int *d_err = nullptr;
    float2 *d_scratch = nullptr;
    float2 *d_rtw = nullptr;
    FftRaggedArgs args{};
    size_t smem = 0;
    unsigned resident = 0;             // CTAs that fit on the device at once
    unsigned grid = 0;
    unsigned split_lg = 13;            // requests of 2^split_lg complex points and more run as phase tasks
    cudaStream_t capture = nullptr;
    cudaGraphExec_t exec = nullptr;
    double algorithmic_bytes = 0;
};

namespace {

void destroy_fft_batch(mufft_gb_fft_batch *b)
{
    if (!b)
        return;
    if (b->device >= 0) {
        DeviceGuard g(b->device);
        if (b->exec)
            cudaGraphExecDestroy(b->exec);
        if (b->capture)
            cudaStreamDestroy(b->capture);
        cudaFree(b->d_reqs);
        cudaFree(b->d_tasks);
        cudaFree(b->d_tab);
        cudaFree(b->d_next);
        cudaFree(b->d_err);
        cudaFree(b->d_scratch);
        cudaFree(b->d_rtw);
    }
    delete b;
}

// Task list for a split size and grid; uploads it and captures the graph
// (counter reset + the persistent launch).
bool fft_batch_build(mufft_gb_fft_batch *b, unsigned split_lg, unsigned grid)
{
    DeviceGuard g(b->device);
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    cudaFree(b->d_tasks);
    cudaFree(b->d_tab);
    cudaFree(b->d_next);
    b->d_tasks = nullptr;
    b->d_tab = nullptr;
    b->d_next = nullptr;
    b->split_lg = split_lg;
    std::vector<FftRaggedReq> reqs = b->sorted;
    std::vector<unsigned> split_ids;
    std::vector<FftRaggedTask> whole;
    std::vector<const float2 *> tab;
    unsigned nsplit = 0;
    // groups of one class, longest first; large requests whole or split
    std::map<std::tuple<unsigned, unsigned, unsigned, unsigned, unsigned>, std::vector<unsigned>> open;
    auto flush = [&](std::vector<unsigned> &grp) {
        whole.push_back(FftRaggedTask{grp[0], kFrGroup, (unsigned short)grp.size(), 0, (unsigned)tab.size()});
        for (unsigned r : grp)
            tab.push_back(reqs[r].in);
        for (unsigned r : grp)
            tab.push_back(reqs[r].out);
        grp.clear();
    };
    for (unsigned i = 0; i < reqs.size(); i++) {
        FftRaggedReq &q = reqs[i];
        if (q.lg > kFrMaxGroupLg) {
            q.split = q.lg >= split_lg ? 1 : 0;
            if (q.split) {
                q.counter = nsplit++;
                split_ids.push_back(i);
            } else {
                whole.push_back(FftRaggedTask{i, 0, kFrWholePhase, 0, 0});
            }
            continue;
        }
        const unsigned gs = fft_ragged_group_size(q.lg);
        std::vector<unsigned> &grp = open[std::make_tuple(q.lg, q.kind, q.inverse, q.half, q.full)];
        grp.push_back(i);
        if (grp.size() == gs)
            flush(grp);
    }
    for (auto &kv : open)
        if (!kv.second.empty())
            flush(kv.second);
    std::stable_sort(whole.begin(), whole.end(),
                     [&](const FftRaggedTask &x, const FftRaggedTask &y) { return reqs[x.req].lg > reqs[y.req].lg; });
    // phase-major over split requests, whole tasks (longest first) in between
    std::vector<FftRaggedTask> tasks;
    size_t w = 0;
    for (unsigned phase = 0; phase < 3; phase++) {
        for (unsigned r : split_ids) {
            unsigned before = 0;
            for (unsigned p = 0; p < phase; p++)
                before += fft_ragged_phase_tasks(reqs[r].lg, p, reqs[r].kind);
            for (unsigned t = 0; t < fft_ragged_phase_tasks(reqs[r].lg, phase, reqs[r].kind); t++)
                tasks.push_back(FftRaggedTask{r, (unsigned short)phase, (unsigned short)t, before, 0});
        }
        const size_t take = phase == 2 ? whole.size() - w : (whole.size() - w) / (3 - phase);
        for (size_t k = 0; k < take; k++, w++)
            tasks.push_back(whole[w]);
    }
    b->next_bytes = (1 + (size_t)nsplit) * sizeof(unsigned);
    if (!cuda_ok(cudaMalloc(&b->d_tasks, std::max<size_t>(1, tasks.size()) * sizeof(FftRaggedTask)),
                 "cudaMalloc(tasks)") ||
        (!tasks.empty() && !cuda_ok(cudaMemcpy(b->d_tasks, tasks.data(), tasks.size() * sizeof(FftRaggedTask),
                                               cudaMemcpyHostToDevice),
                                    "cudaMemcpy(tasks)")) ||
        !cuda_ok(cudaMalloc(&b->d_tab, std::max<size_t>(1, tab.size()) * sizeof(float2 *)), "cudaMalloc(tables)") ||
        (!tab.empty() && !cuda_ok(cudaMemcpy(b->d_tab, tab.data(), tab.size() * sizeof(float2 *),
                                             cudaMemcpyHostToDevice),
                                  "cudaMemcpy(tables)")) ||
        !cuda_ok(cudaMemcpy(b->d_reqs, reqs.data(), reqs.size() * sizeof(FftRaggedReq), cudaMemcpyHostToDevice),
                 "cudaMemcpy(requests)") ||
        !cuda_ok(cudaMalloc(&b->d_next, b->next_bytes), "cudaMalloc(counters)"))
        return false;
    b->args.reqs = b->d_reqs;
    b->args.tasks = b->d_tasks;
    b->args.count = (unsigned)tasks.size();
    b->args.next = b->d_next;
    b->args.err = b->d_err;
    b->args.tab = b->d_tab;
    b->grid = std::max(1u, std::min<unsigned>(grid, (unsigned)tasks.size()));
    void *kargs[] = {&b->args};
    cudaGraph_t gr = nullptr;
    bool ok = cuda_ok(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "capture") &&
              cuda_ok(cudaMemsetAsync(b->d_next, 0, b->next_bytes, b->capture), "cudaMemsetAsync") &&
              cuda_ok(cudaLaunchKernel(fft_ragged_fn(), dim3(b->grid), dim3(fft_ragged_threads()), kargs, b->smem,
                                       b->capture),
                      "kernel launch");
    const cudaError_t ce = cudaStreamEndCapture(b->capture, &gr);
    ok = ok && cuda_ok(ce, "capture") && cuda_ok(cudaGraphInstantiate(&b->exec, gr, 0), "cudaGraphInstantiate");
    if (gr)
        cudaGraphDestroy(gr);
    return ok;
}

}  // namespace

extern "C" {

mufft_gb_fft_batch *mufft_gb_create_fft_batch(const mufft_gb_fft_request *requests, unsigned count, unsigned flags,
                                              const mufft_gb_options *opts)
{
    t_err = 0;
    mufft_gb_options o;
    if (!public_options(opts, &o))
        return nullptr;
    if (!requests || count == 0) {
        set_error(MUFFT_GB_ERR_INVALID, "no requests");
        return nullptr;
    }
    std::vector<FftRaggedReq> reqs(count);
    std::vector<size_t> scratch_off(count, (size_t)-1);
    size_t scratch_elems = 0;
    bool need[kFrMaxLg + 1] = {};
    double algo = 0;
    const unsigned allowed = MUFFT_FLAG_ZERO_PAD_UPPER_HALF | MUFFT_FLAG_FULL_R2C | MUFFT_FLAG_CPU_NO_SIMD;
    for (unsigned i = 0; i < count; i++) {
        const mufft_gb_fft_request &r = requests[i];
        const bool zp = (r.flags & MUFFT_FLAG_ZERO_PAD_UPPER_HALF) != 0;
        const bool full = (r.flags & MUFFT_FLAG_FULL_R2C) != 0;
        if (r.kind < 0 || r.kind > 2 || !is_pow2(r.N) || r.N == 1 || (r.kind != 0 && r.N < 4) || !r.input ||
            !r.output || (r.flags & ~allowed) ||
            (r.kind == 0 && r.direction != MUFFT_FORWARD && r.direction != MUFFT_INVERSE) ||
            ((uintptr_t)r.input & 7) || ((uintptr_t)r.output & 7)) {
            set_error(MUFFT_GB_ERR_INVALID,
                      "request %u: kind 0..2, N a power of two (>= 4 for real kinds), a direction of +-1 for c2c, "
                      "8-byte aligned buffers and only the zero-pad / full-output flags",
                      i);
            return nullptr;
        }
        const unsigned L = r.kind == 0 ? r.N : r.N / 2;
        const unsigned lg = ilog2u(L);
        if (lg > kFrMaxLg) {
            set_error(MUFFT_GB_ERR_UNSUPPORTED, "request %u: N=%u beyond the ragged range (%u complex points)", i,
                      r.N, 1u << kFrMaxLg);
            return nullptr;
        }
        FftRaggedReq &q = reqs[i];
        q.in = (const float2 *)r.input;
        q.out = (float2 *)r.output;
        q.lg = lg;
        q.kind = (unsigned)r.kind;
        q.inverse = (r.kind == 0 && r.direction == MUFFT_INVERSE) ? 1 : 0;
        q.half = zp ? 1 : 0;
        q.full = (r.kind == 1 && full) ? 1 : 0;
        need[lg] = true;
        if (lg > kFrMaxGroupLg) {
            scratch_off[i] = scratch_elems;
            scratch_elems += ((size_t)L + 31) & ~(size_t)31;  // 256-byte aligned slots
        }
        // algorithmic bytes: read the input once, write the output once
        const double in_b = r.kind == 0 ? 8.0 * (zp ? r.N / 2 : r.N)
                                        : (r.kind == 1 ? 4.0 * (zp ? r.N / 2 : r.N) : 8.0 * (r.N / 2 + 1));
        const double out_b = r.kind == 0 ? 8.0 * r.N : (r.kind == 1 ? 8.0 * (full ? r.N : r.N / 2 + 1) : 4.0 * r.N);
        algo += in_b + out_b;
    }
    int dev;
    if (!device_prepare(&dev))
        return nullptr;
    mufft_gb_fft_batch *b = new mufft_gb_fft_batch();
    b->device = dev;
    b->count = count;
    b->algorithmic_bytes = algo;
    FftRaggedArgs &args = b->args;
    // per length: r2c fix-up twiddles then c2r ones, FP64 then rounded (fft.c:441-455)
    std::vector<float2> rtw;
    for (unsigned lg = 0; lg <= kFrMaxLg; lg++) {
        args.rtw_off[lg] = (unsigned)rtw.size();
        if (!need[lg])
            continue;
        std::vector<float2> f = r2c_twiddles(MUFFT_FORWARD, 1u << lg), iv = r2c_twiddles(MUFFT_INVERSE, 1u << lg);
        rtw.insert(rtw.end(), f.begin(), f.end());
        rtw.insert(rtw.end(), iv.begin(), iv.end());
    }
    b->d_rtw = upload(rtw);
    if (!b->d_rtw ||
        (scratch_elems && !cuda_ok(cudaMalloc(&b->d_scratch, scratch_elems * sizeof(float2)), "cudaMalloc(scratch)")) ||
        !cuda_ok(cudaMalloc(&b->d_reqs, count * sizeof(FftRaggedReq)), "cudaMalloc(requests)") ||
        !cuda_ok(cudaMalloc(&b->d_err, sizeof(int)), "cudaMalloc(err)") ||
        !cuda_ok(cudaMemset(b->d_err, 0, sizeof(int)), "cudaMemset(err)") ||
        !cuda_ok(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), "cudaStreamCreate")) {
        destroy_fft_batch(b);
        return nullptr;
    }
    for (unsigned i = 0; i < count; i++)
        if (scratch_off[i] != (size_t)-1)
            reqs[i].scratch = b->d_scratch + scratch_off[i];
    // longest first (by points x log2 points), so the largest requests start at once
    std::vector<unsigned> order(count);
    for (unsigned i = 0; i < count; i++)
        order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](unsigned x, unsigned y) { return reqs[x].lg > reqs[y].lg; });
    b->sorted.resize(count);
    for (unsigned i = 0; i < count; i++)
        b->sorted[i] = reqs[order[i]];
    b->smem = fft_ragged_smem();
    args.tw = g_dev[dev].tw;
    args.rtw = b->d_rtw;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (!cuda_ok(cudaFuncSetAttribute(fft_ragged_fn(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem),
                 "cudaFuncSetAttribute") ||
        !cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fft_ragged_fn(), fft_ragged_threads(),
                                                               b->smem),
                 "occupancy")) {
        destroy_fft_batch(b);
        return nullptr;
    }
    b->resident = (unsigned)(sms * std::max(per_sm, 1));
    // Split size from the options (default: every request of 8192 points and
    // more as phase tasks), the persistent grid filling the device.
    // MUFFT_GB_FLAG_AUTOTUNE times the split sizes (8192 .. 65536 points, or
    // none) and grids of one to all resident CTAs per SM, and keeps the fastest.
    unsigned best_lg = o.fft_split ? ilog2u(o.fft_split) : kFrMaxLg + 1, best_grid = b->resident;
    if (flags & MUFFT_GB_FLAG_AUTOTUNE) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        bool ok = cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") && cuda_ok(cudaEventCreate(&e1), "cudaEventCreate");
        double best = INFINITY;
        for (unsigned lg = kFrMaxGroupLg + 1; ok && lg <= kFrMaxLg + 1; lg++)
            for (int per = std::max(per_sm, 1); ok && per >= 1; per = per > 1 ? per / 2 : 0) {
                const unsigned grid = (unsigned)(sms * per);
                if (!fft_batch_build(b, lg, grid)) {
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
                    best_lg = lg;
                    best_grid = grid;
                }
            }
        if (e0)
            cudaEventDestroy(e0);
        if (e1)
            cudaEventDestroy(e1);
        if (!ok) {
            destroy_fft_batch(b);
            return nullptr;
        }
    }
    if (!fft_batch_build(b, best_lg, best_grid)) {
        destroy_fft_batch(b);
        return nullptr;
    }
    return b;
}

int mufft_gb_execute_fft_batch(mufft_gb_fft_batch *batch, void *stream)
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

int mufft_gb_fft_batch_status(mufft_gb_fft_batch *batch)
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

int mufft_gb_fft_batch_describe(const mufft_gb_fft_batch *batch, char *buf, size_t size)
{
    if (!batch || !buf || !size) {
        set_error(MUFFT_GB_ERR_INVALID, "null batch or buffer");
        return MUFFT_GB_ERR_INVALID;
    }
    snprintf(buf, size, "requests=%u tasks=%u split=%u grid=%u resident=%u algorithmic_bytes=%.0f", batch->count,
             batch->args.count, batch->split_lg > kFrMaxLg ? 0u : 1u << batch->split_lg, batch->grid, batch->resident,
             batch->algorithmic_bytes);
    return MUFFT_GB_OK;
}

void mufft_gb_free_fft_batch(mufft_gb_fft_batch *batch) { destroy_fft_batch(batch); }

}  // extern "C"
