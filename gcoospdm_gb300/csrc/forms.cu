// forms.cu -- dispatch of the reduced-precision forms (gcoo_spdm_ex) to an
// engine: the tcgen05 tensor-core engine (spdm_tc.cu) where the matrix's
// entries densify into 16-column tiles of its row panels (256 rows for BF16
// and FP8-B, 128 for split-BF16), the FMA engine (spdm_lowp.cu) elsewhere. FP8-B on the tensor engine: B quantized to E4M3 with
// power-of-two column scales and multiplied as exact BF16 values (kind::f16
// needs both operands 16-bit), A in BF16 as for the BF16 form.
#include "handle.hpp"

namespace gcoo {

// spdm_lowp.cu
int lowp_vec(gcoo_precision prec);
gcoo_status lowp_prepare(gcoo_handle *h, int64_t n, gcoo_precision prec);
gcoo_status lowp_convert_b(gcoo_handle *h, const float *dB, int64_t n, gcoo_precision prec, cudaStream_t st);
gcoo_status lowp_spdm(gcoo_handle *h, int64_t n, float *dC, gcoo_precision prec, cudaStream_t st);
// spdm_tc.cu
gcoo_status tc_build_plan(gcoo_handle *h, bool split, cudaStream_t st);
double tc_density(const gcoo_handle *h);
gcoo_status tc_prepare_b(gcoo_handle *h, int64_t n, bool fp8);
gcoo_status tc_spdm(gcoo_handle *h, const float *dB, int64_t n, float *dC, bool fp8, cudaStream_t st);

// Entries per stored tile slot above which the tensor engine wins: a tile
// costs its MMAs whatever its fill, which the tensor pipe runs at more than
// 16x the rate the FMA pipes serve one entry per output column.
constexpr double kTensorDensity = 1.0 / 16.0;

bool form_uses_tensor(gcoo_handle *h, gcoo_precision prec)
{
    if (prec != GCOO_PREC_BF16 && prec != GCOO_PREC_SPLIT_BF16 && prec != GCOO_PREC_FP8_B)
        return false;
    if (h->p.engine == GCOO_ENGINE_CUDA_CORE)
        return false;
    if (h->p.engine == GCOO_ENGINE_TENSOR)
        return true;
    if (tc_build_plan(h, prec == GCOO_PREC_SPLIT_BF16, nullptr) != GCOO_SUCCESS)
        return false;
    return tc_density(h) >= kTensorDensity;
}

gcoo_status run_form(gcoo_handle *h, const float *dB, int64_t n, float *dC, gcoo_precision prec, cudaStream_t st,
                     bool prepare_only)
{
    const bool aligned = prepare_only || ((reinterpret_cast<uintptr_t>(dB) & 15) == 0 &&
                                          (reinterpret_cast<uintptr_t>(dC) & 15) == 0);
    bool tensor = false;
    if (prec == GCOO_PREC_BF16 || prec == GCOO_PREC_SPLIT_BF16 || prec == GCOO_PREC_FP8_B) {
        if (h->p.engine == GCOO_ENGINE_TENSOR || h->p.engine == GCOO_ENGINE_AUTO) {
            gcoo_status s = tc_build_plan(h, prec == GCOO_PREC_SPLIT_BF16, st);
            if (s != GCOO_SUCCESS)
                return s;
            tensor = h->p.engine == GCOO_ENGINE_TENSOR || tc_density(h) >= kTensorDensity;
        }
    }
    if (tensor) {
        if (n % 16 != 0 || !aligned)
            return fail(GCOO_ERROR_UNSUPPORTED, "the tensor-core engine needs n % 16 == 0 and 16-byte aligned B and C");
        const bool fp8 = prec == GCOO_PREC_FP8_B;
        gcoo_status s = tc_prepare_b(h, n, fp8);
        if (s != GCOO_SUCCESS || prepare_only)
            return s;
        return tc_spdm(h, dB, n, dC, fp8, st);
    }
    const int V = lowp_vec(prec);
    if (n % V != 0 || !aligned)
        return fail(GCOO_ERROR_UNSUPPORTED, "this form on the FMA engine needs n % " + std::to_string(V) +
                                                " == 0 and 16-byte aligned B and C");
    gcoo_status s = lowp_prepare(h, n, prec);
    if (s != GCOO_SUCCESS || prepare_only)
        return s;
    s = lowp_convert_b(h, dB, n, prec, st);
    if (s != GCOO_SUCCESS)
        return s;
    return lowp_spdm(h, n, dC, prec, st);
}

} // namespace gcoo
