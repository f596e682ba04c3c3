// Host build of the power-of-two pass kernel's launch tables for one
// arithmetic (EMU_ARITH: 0 FP64, 1 double-float FP64, 2 FP32, 3 double-float
// FP32), for log2 L = 1..8 and every lines-per-CTA value; longer lines are
// not built for the host (the dispatch then reports them unsupported).
#include "fft_pass.cuh"

namespace tfft {

#if EMU_ARITH == 0
using EA = ArithF64;
#elif EMU_ARITH == 1
using EA = ArithDF64;
#elif EMU_ARITH == 2
using EA = ArithF32;
#else
using EA = ArithDF32;
#endif

static constexpr auto kTable = range_table<EA, 1, 8>(std::make_integer_sequence<int, 8>{});

static LaunchFn emu_find(int log_l, int log_b)
{
    if (log_l < 1 || log_l > 8 || log_b < 0 || log_b > kMaxLogB) return nullptr;
    return kTable.fn[log_l][log_b];
}

#if EMU_ARITH == 0
LaunchFn launcher_f64_lo(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_f64_hi(int, int) { return nullptr; }
#elif EMU_ARITH == 1
LaunchFn launcher_df64_0(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_df64_1(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_df64_2(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_df64_3(int, int) { return nullptr; }
LaunchFn launcher_df64_4(int, int) { return nullptr; }
LaunchFn launcher_df64_5(int, int) { return nullptr; }
#elif EMU_ARITH == 2
LaunchFn launcher_f32_lo(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_f32_hi(int, int) { return nullptr; }
#else
LaunchFn launcher_df32_0(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_df32_1(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_df32_2(int l, int b) { return emu_find(l, b); }
LaunchFn launcher_df32_3(int, int) { return nullptr; }
LaunchFn launcher_df32_4(int, int) { return nullptr; }
LaunchFn launcher_df32_5(int, int) { return nullptr; }
#endif

} // namespace tfft
