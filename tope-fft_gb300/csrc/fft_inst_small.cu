/* Pass-kernel instantiations with 4 points per thread (radix-4 stages) for
 * small transforms in FP64 storage: native FP64 and double-float, log2 L =
 * 2..7, lines per CTA with log2 L + log2 B <= 12 (at most 1024 threads). */
#include "fft_pass.cuh"

namespace tfft {
namespace {

constexpr int kLo = 2, kHi = 7;

template <class A, int LOG_L, int LOG_B>
constexpr LaunchFn pick4()
{
    if constexpr (LOG_L + LOG_B <= 12) return &launch_pass<A, LOG_L, LOG_B, 4>;
    else return nullptr;
}

template <class A, int LOG_L, int... LB>
constexpr void fill_row4(LaunchFn *row, std::integer_sequence<int, LB...>)
{
    ((row[LB] = pick4<A, LOG_L, LB>()), ...);
}

template <class A, int... I>
struct Table4 {
    LaunchFn fn[kHi + 1][kMaxLogB + 1];
    constexpr Table4() : fn{}
    {
        (fill_row4<A, kLo + I>(fn[kLo + I], std::make_integer_sequence<int, kMaxLogB + 1>{}), ...);
    }
};

template <class A, int... I>
constexpr Table4<A, I...> table4(std::integer_sequence<int, I...>)
{
    return Table4<A, I...>();
}

const auto g_f64 = table4<ArithF64>(std::make_integer_sequence<int, kHi - kLo + 1>{});
const auto g_df64 = table4<ArithDF64>(std::make_integer_sequence<int, kHi - kLo + 1>{});

}  // namespace

LaunchFn launcher_small(int arith, int log_l, int log_b)
{
    if (log_l < kLo || log_l > kHi || log_b < 0 || log_b > kMaxLogB) return nullptr;
    if (arith == TFFT_ARITH_F64) return g_f64.fn[log_l][log_b];
    if (arith == TFFT_ARITH_DF64) return g_df64.fn[log_l][log_b];
    return nullptr;
}

}  // namespace tfft
