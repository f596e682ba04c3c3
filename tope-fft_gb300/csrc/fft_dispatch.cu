/*
 * Launch dispatch of the pass kernel: (arithmetic, log2 L, lines per CTA)
 * -> the instantiation compiled in one of the fft_inst_*.cu units.
 * Valid shapes: L = 2^0..2^13, B = 1..32 with L*B <= 8192 (at most 512
 * threads and 136 KB of shared memory per CTA).
 */
#include "fft_pass.cuh"

namespace tfft {

static int ilog2_exact(int v)
{
    int l = 0;
    while ((1 << l) < v) l++;
    return (1 << l) == v ? l : -1;
}

static LaunchFn find(int log_l, int b_tile, int arith, int ept)
{
    const int log_b = ilog2_exact(b_tile);
    if (ept == 4) return log_b < 0 ? nullptr : launcher_small(arith, log_l, log_b);
    if (ept != 0 && ept != 16) return nullptr;
    /* the tensor form fixes its lines per CTA (up to 256 for L = 16) */
    if (arith == TFFT_ARITH_TC && log_l >= 4)
        return log_l <= 13 && b_tile == tfft_tc_b_tile(log_l) ? launcher_tc(log_l) : nullptr;
    if (log_l < 0 || log_l > TFFT_MAX_LOG_L || log_b < 0 || log_b > kMaxLogB) return nullptr;
    if (log_l > TFFT_MAX_LOG_L_ARITH(arith)) return nullptr;
    if (arith == TFFT_ARITH_F64)
        return log_l <= 9 ? launcher_f64_lo(log_l, log_b) : launcher_f64_hi(log_l, log_b);
    if (arith == TFFT_ARITH_F32)
        return log_l <= 9 ? launcher_f32_lo(log_l, log_b) : launcher_f32_hi(log_l, log_b);
    /* lines of the tensor form below 16 points: the accurate form's kernel */
    if (arith == TFFT_ARITH_TC) arith = TFFT_ARITH_DF32;
    if (arith == TFFT_ARITH_DF64) {
        if (log_l <= 4) return launcher_df64_0(log_l, log_b);
        if (log_l <= 6) return launcher_df64_1(log_l, log_b);
        if (log_l <= 8) return launcher_df64_2(log_l, log_b);
        if (log_l <= 9) return launcher_df64_3(log_l, log_b);
        if (log_l <= 11) return launcher_df64_4(log_l, log_b);
        return launcher_df64_5(log_l, log_b);
    }
    if (arith == TFFT_ARITH_DF32) {
        if (log_l <= 4) return launcher_df32_0(log_l, log_b);
        if (log_l <= 6) return launcher_df32_1(log_l, log_b);
        if (log_l <= 8) return launcher_df32_2(log_l, log_b);
        if (log_l <= 9) return launcher_df32_3(log_l, log_b);
        if (log_l <= 11) return launcher_df32_4(log_l, log_b);
        return launcher_df32_5(log_l, log_b);
    }
    return nullptr;
}

} // namespace tfft

extern "C" int tfft_pass_supported(int log_l, int b_tile, int arith, int ept)
{
    return tfft::find(log_l, b_tile, arith, ept) != nullptr;
}

extern "C" int tfft_pass_bulk_capable(int log_l, int b_tile, int arith, int ept)
{
    /* bulk_capable() of fft_pass.cuh for the shapes find() launches with the
     * ordinary pass kernel */
    if (arith == TFFT_ARITH_TC || (ept != 0 && ept != 16)) return 0;
    if (b_tile < 8 || log_l < 5 || (int64_t(TFFT_ELEM_BYTES(arith)) << log_l) < 512) return 0;
    return tfft::find(log_l, b_tile, arith, ept) != nullptr;
}

extern "C" int tfft_launch_pass(const tfft_pass *p, void *stream)
{
    if (p->len) return tfft::launch_mixed(*p, (cudaStream_t)stream);
    tfft::LaunchFn f = tfft::find(p->log_l, p->b_tile, p->arith, p->ept);
    if (!f) return (int)cudaErrorInvalidValue;
    return f(*p, (cudaStream_t)stream);
}
