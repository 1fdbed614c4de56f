// Convolution plans: the reference's mufft_create_plan_conv /
// mufft_execute_conv_input / _output (fft.c:565-624, 794-809) -- the spectral
// multiply is fused into the inverse transform's loads -- plus
// mufft_get_convolve_func, the batched output form and the adjoints.
#include <cstdio>

#include "host.h"
#include "misc_kernels.h"

using namespace mgb;

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
    // options of the creation call, applied to the plans made later too
    PlanOptions opts;
    bool has_opts = false;
    const PlanOptions *options() const { return has_opts ? &opts : nullptr; }
};

extern "C" {

mufft_plan_conv *mufft_create_plan_conv(unsigned N, unsigned flags, unsigned method)
{
    return mufft_gb_create_plan_conv(N, flags, method, nullptr);
}

mufft_plan_conv *mufft_gb_create_plan_conv(unsigned N, unsigned flags, unsigned method, const mufft_gb_options *opts)
{
    t_err = 0;
    PlanOptions o;
    if (opts && !convert_options(opts, &o))
        return nullptr;
    if (!is_pow2(N) || N == 1) {
        set_error(MUFFT_GB_ERR_INVALID, "N=%u is not a power of two >= 2", N);
        return nullptr;
    }
    mufft_plan_conv *c = new mufft_plan_conv();
    c->N = N;
    c->method = method;
    c->opts = o;
    c->has_opts = opts != nullptr;
    OptionsScope scope(c->options());
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
    OptionsScope scope(plan->options());
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
    OptionsScope scope(plan->options());
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
    OptionsScope scope(plan->options());
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
    OptionsScope scope(plan->options());
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

