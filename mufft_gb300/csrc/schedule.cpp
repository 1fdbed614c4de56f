// The launch schedule of a transform ("passes"): how a plan's kernels are
// launched, described and built.
//
// Where the reference builds a list of CPU passes (fft.c:325-435), this file
// builds a list of GPU launches:
//   - complex length M <= 16384: one tile-FFT launch (one HBM read + write per
//     transform), with the r2c/c2r fix-up and the convolution multiply fused
//     into its load or store phase;
//   - M > 16384: a four-step pair, M = N1 x N2 (column FFTs of length N1 with
//     the W_M^(k1*n2) twiddle fused into their stores, then row FFTs of length
//     N2 with transposed stores into natural order), or from 2^22 points three
//     levels of smaller tiles.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "host.h"
#include "misc_kernels.h"

namespace mgb {

static const void *pick(Role r, const Buffers &b)
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

static EncodeTiledFn encode_tiled()
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
static bool tma_map_for(const Pass &p, const float2 *in, CUtensorMap *map)
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

// Dynamic shared memory of a tile launch: the four-step twiddle region only
// where an epilogue reads it, at least the resident-CTA cap's request.
static size_t tile_launch_smem(const Pass &p)
{
    const TileArgs &a = p.a;
    return std::max((a.tw_lo || a.tw_colpow || a.tw_by_y) ? p.k->smem : p.k->smem_ex, p.smem_min);
}

// A row tile with a c2r fix-up prologue over whole rows runs as its variant
// that stages each row in shared memory.
static bool uses_c2r_rows(const Pass &p)
{
    const TileArgs &a = p.a;
    return p.k->fn_c2r && (a.prologue == PRO_C2R || a.prologue == PRO_MUL_C2R) && a.mirror_ldist == 0 &&
           a.mirror_len == p.k->L && !a.half && a.in_stride == 1;
}

cudaError_t run_passes(const std::vector<Pass> &ps, const Buffers &b, cudaStream_t st, size_t first, size_t count)
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
            if (p.pt) {
                unsigned tiles_x = p.grid.x, ntiles = p.grid.x * p.grid.y;
                void *pargs[] = {&a, &tiles_x, &ntiles};
                cudaError_t e = cudaLaunchKernel(p.pt->fn, dim3(std::min(ntiles, p.pt_grid)), dim3(p.pt->threads),
                                                 pargs, tile_launch_smem(p), st);
                if (e != cudaSuccess)
                    return e;
                continue;
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
            const size_t smem = tile_launch_smem(p);
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
                e = cudaLaunchKernel(uses_c2r_rows(p) ? p.k->fn_c2r : p.k->fn, p.grid, dim3(p.k->threads), args, smem,
                                     st);
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

static const char *pro_name(int p)
{
    static const char *n[] = {"plain", "c2r", "mul", "mul_c2r"};
    return (p >= 0 && p < 4) ? n[p] : "?";
}
static const char *epi_name(int e)
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
                     i ? "; " : "", p.tk ? (p.tk->nbuf == 2 ? "+tma2" : "+tma1") : (p.sk ? "+stream" : (p.pt ? "+persistent" : "")), p.k->L, p.k->R, p.k->C, p.k->Q, p.k->lmap ? "across" : "along",
                     p.k->smap ? "across" : "along", p.sk ? p.sk_grid : (p.pt ? std::min(p.grid.x * p.grid.y, p.pt_grid) : p.grid.x), p.pt ? 1u : p.grid.y, p.k->threads, std::max(p.k->smem, p.smem_min),
                     pro_name(p.a.prologue), p.a.half ? "+half" : "", epi_name(p.a.epilogue),
                     p.a.epilogue != EPI_TWIDDLE ? ""
                     : (p.a.tw_by_y ? "/by_row" : (p.a.tw_colpow ? "/colpow" : (p.a.tw_lo ? "/table" : "/sincos"))),
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
        if (p.type == PASS_TILE && p.a.l2) {
            // L2 policy: loads evict-first, stores evict-last / evict-first, input discarded
            s += " l2=";
            s += (p.a.l2 & L2_LOAD_FIRST) ? "F" : "";
            s += (p.a.l2 & L2_STORE_LAST) ? "L" : "";
            s += (p.a.l2 & L2_STORE_FIRST) ? "S" : "";
            s += (p.a.l2 & L2_DISCARD_IN) ? "D" : "";
        }
    }
    return s;
}

void PlanResources::release()
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

static bool use_twiddle_table(const TileKernel *k)
{
    const int t = opt_twiddle();
    return k->has_thi && t == 1;
}

// Column powers (mode 2, and the automatic choice wherever the tile has the
// shared-memory region): the twiddles of a column are W^(col*base) of each
// thread times R per-column powers computed once per tile.
static bool use_colpow(const TileKernel *k)
{
    const int t = opt_twiddle();
    return k->has_thi && (t == 2 || t < 0);
}

// W_M^(k*c) for k < L, c < C: the per-column half of a four-step twiddle.
static bool upload_twlo(unsigned L, int C, unsigned long long M, float2 *&dst)
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
static Pass column_pass(const TileKernel *k, const float2 *tw, unsigned L, unsigned ncols, long long stride,
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

// Gives every single-CTA tile pass whose tile has a persistent variant that
// variant: a grid of SMs x resident CTAs walking the pass's tiles (not for
// c2r row tiles, which stage their rows in tile_fft_c2r_rows).
bool attach_persist(std::vector<Pass> &ps, bool dry, int device)
{
    if (opt_persist() != 1)
        return true;
    for (Pass &p : ps) {
        if (p.type != PASS_TILE || !p.k || p.k->Q != 1 || p.tk || p.sk || p.grid.z > 1 || uses_c2r_rows(p))
            continue;
        const PersistTileKernel *pt = find_persist(p.k->L, p.k->R, p.k->C, p.k->lmap, p.k->smap);
        if (!pt)
            continue;
        int sms = 152, per_sm = 1;
        if (!dry) {
            // the kernel's limit is the device's opt-in maximum, so that no
            // plan created later lowers it under an earlier plan's launch
            // (with or without the twiddle region, any resident-CTA cap)
            const size_t smem = tile_launch_smem(p);
            int limit = 232448;
            cudaDeviceGetAttribute(&limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            if (!cuda_ok(cudaFuncSetAttribute(pt->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, limit),
                         "cudaFuncSetAttribute(persist)") ||
                !cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pt->fn, pt->threads, smem),
                         "occupancy(persist)"))
                return false;
            if (per_sm < 1)
                continue;
        }
        p.pt = pt;
        p.pt_grid = (unsigned)(sms * per_sm);
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
        if (p.type != PASS_TILE || !p.k || p.k->Q != 1 || p.tk || p.sk || p.pt)
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
        if (opt_l2() == 1) {
            // keep the intermediate in L2 as far as it fits: A streams its
            // input and marks its stores evict-last, B (in place) keeps them
            // so, C drops each row from L2 once read (its rows are 128-byte
            // aligned: N3 >= 16 points at offsets of N3 points) and streams
            // its output unless an r2c fix-up reads it next
            pa.a.l2 = L2_LOAD_FIRST | L2_STORE_LAST;
            pb.a.l2 = L2_STORE_LAST;
            pc.a.l2 = (N3 >= 16 ? L2_DISCARD_IN : 0) | (r2c ? 0 : L2_STORE_FIRST);
            out[out.size() - 2].a.l2 = pa.a.l2;
            out[out.size() - 1].a.l2 = pb.a.l2;
        }
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
    constexpr size_t kL2HintMaxScratch = (size_t)128 << 20;  // about the L2 of a GB300
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
    if (opt_l2() == 1 && (size_t)M * s.batch * sizeof(float2) <= kL2HintMaxScratch) {
        // the intermediate as in the three-level schedule: kept in L2 by the
        // first pass, dropped without write-back once the second has read it
        // (rows of N2 >= 128 points, 128-byte aligned).  Only where it about
        // fits: for larger batches the hints measured slower (c2c 2^21 x 64
        // 917 -> 957 us, 2^20 x 128 857 -> 898 us, 2^21 x 16 246 -> 253 us)
        // against 2^16 x 256 94.2 -> 89.6 us and r2c 2^21 x 8 101.6 -> 94.0 us.
        out.back().a.l2 = L2_LOAD_FIRST | L2_STORE_LAST;
        p2.a.l2 = L2_DISCARD_IN | (r2c ? 0 : L2_STORE_FIRST);
    }
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

void Staging::release()
{
    cudaFree(in);
    cudaFree(out);
    cudaFree(in2);
    in = out = in2 = nullptr;
    in_bytes = out_bytes = in2_bytes = 0;
}

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

}  // namespace mgb
