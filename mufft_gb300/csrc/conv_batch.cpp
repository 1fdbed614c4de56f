// Ragged batched convolution, host side: the request table, the task order
// of the persistent kernel (conv_ragged.cu), the class pipelines and the
// CUDA graph that replays a batch.
#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>

#include "conv_ragged.h"
#include "host.h"

using namespace mgb;

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
                                                unsigned flags, const mufft_gb_options *opts)
{
    t_err = 0;
    mufft_gb_options o;
    if (!public_options(opts, &o))
        return nullptr;
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
    // Defaults (mufft_gb_options_init), measured on the 512-request mix of
    // 2^8..2^16 points: splitting the 65536-point requests took the batch from
    // 0.19 to 0.177 ms (splitting 32768 and 16384 as well cost more in task
    // overhead than it gained: 0.226, 0.259 ms); class pipelines from 65536 /
    // 32768 / 16384 points then gave 0.152 / 0.148 / 0.146 ms.
    unsigned best_lg = o.conv_split ? ilog2u(o.conv_split) : 17u;
    unsigned best_class = o.conv_classes ? ilog2u(o.conv_classes) : 17u, best_small = 0;
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
        Cand best_c{best_lg, best_class, 0};
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
