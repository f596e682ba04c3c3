/*
 * Native-FP64 instantiations of the pass kernel and the launch dispatch for
 * every arithmetic.  Valid shapes: L = 2^0..2^13, B = 1..32 with L*B <= 8192
 * (at most 512 threads and 136 KB of shared memory per CTA).
 */
#include <utility>

#include "fft_pass.cuh"

namespace tfft {

using LaunchFn = int (*)(const tfft_pass &, cudaStream_t);

constexpr int kMaxLogB = 5;

template <class A, int LOG_L, int LOG_B>
constexpr LaunchFn pick()
{
    if constexpr (LOG_L + LOG_B <= 13) return &launch_pass<A, LOG_L, LOG_B>;
    else return nullptr;
}

template <class A, int LOG_L, int... LB>
constexpr void fill_row(LaunchFn *row, std::integer_sequence<int, LB...>)
{
    ((row[LB] = pick<A, LOG_L, LB>()), ...);
}

template <class A, int... LL>
struct Table {
    LaunchFn fn[TFFT_MAX_LOG_L + 1][kMaxLogB + 1];
    constexpr Table() : fn{}
    {
        (fill_row<A, LL>(fn[LL], std::make_integer_sequence<int, kMaxLogB + 1>{}), ...);
    }
};

template <class A, int... LL>
constexpr Table<A, LL...> make_table(std::integer_sequence<int, LL...>)
{
    return Table<A, LL...>();
}

static const auto g_f64 = make_table<ArithF64>(std::make_integer_sequence<int, TFFT_MAX_LOG_L + 1>{});

/* defined in fft_pass_df64.cu */
LaunchFn df64_launcher(int log_l, int log_b);

static int ilog2_exact(int v)
{
    int l = 0;
    while ((1 << l) < v) l++;
    return (1 << l) == v ? l : -1;
}

static LaunchFn find(int log_l, int b_tile, int arith)
{
    const int log_b = ilog2_exact(b_tile);
    if (log_l < 0 || log_l > TFFT_MAX_LOG_L || log_b < 0 || log_b > kMaxLogB) return nullptr;
    if (arith == TFFT_ARITH_F64) return g_f64.fn[log_l][log_b];
    if (arith == TFFT_ARITH_DF64) return df64_launcher(log_l, log_b);
    return nullptr;
}

} // namespace tfft

extern "C" int tfft_pass_supported(int log_l, int b_tile, int arith)
{
    return tfft::find(log_l, b_tile, arith) != nullptr;
}

extern "C" int tfft_launch_pass(const tfft_pass *p, void *stream)
{
    tfft::LaunchFn f = tfft::find(p->log_l, p->b_tile, p->arith);
    if (!f) return (int)cudaErrorInvalidValue;
    if (p->n[0] % p->b_tile) return (int)cudaErrorInvalidValue;
    return f(*p, (cudaStream_t)stream);
}
