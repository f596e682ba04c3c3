// The pass kernel's shared-memory exchange layout (sidx in
// tope-fft_gb300/csrc/fft_pass.cuh) against a bank model, on the host.
// For every element size (8 bytes: FP32 complex; 16 bytes: FP64 complex and
// double-float pairs), every line length 2^5 .. 2^13 and every tile of B
// lines with at least one warp, it replays the Stockham stages' reads
// (p = j + q * TPL) and writes (p = o + r * NS) of each warp with the kernel's
// own index function, and counts the shared-memory wavefronts: requests are
// served in 128-byte phases (16 threads of 8-byte or 8 threads of 16-byte
// accesses), and a phase takes as many wavefronts as the largest number of
// distinct 4-byte words any of the 32 banks holds.  A layout is conflict-free
// when every request takes its minimum (2 or 4 phases of one wavefront).
// It also checks that the layout is a one-to-one map into the exchange
// buffer (pass_smem_bytes), and the reads of tiles staged by bulk copies
// (slots of bulk_slot_bytes per line).  Prints one line per shape; exit status 0 when
// every shape is conflict-free and one-to-one.
#include <cstdint>
#include <cstdio>
#include <set>
#include <utility>
#include <vector>

#include "cuda_runtime.h"
#include "fft_pass.cuh"

using namespace tfft;

struct Count {
    long waves = 0, ideal = 0;
};

/* wavefronts of one warp's request: byte addresses of 32 threads */
static void add_request(const std::vector<long> &addr, int es, Count &c)
{
    const int per = es == 8 ? 16 : 8;
    for (int ph = 0; ph < 32; ph += per) {
        std::set<long> words[32];
        for (int t = ph; t < ph + per; t++)
            for (int w = 0; w < es / 4; w++) {
                const long word = addr[t] / 4 + w;
                words[word % 32].insert(word);
            }
        size_t m = 0;
        for (auto &s : words) m = s.size() > m ? s.size() : m;
        c.waves += (long)m;
        c.ideal += 1;
    }
}

template <int ES, int LOG_L, int B>
static bool check()
{
    using SH = Shape<LOG_L, 16>;
    constexpr int L = SH::L, E = SH::E, TPL = SH::TPL, NT = TPL * B;
    if constexpr (NT < 32 || TPL < 2) {
        return true;
    } else {
        /* one-to-one into the buffer */
        constexpr size_t cap = ((size_t)L + (L >> 4)) * B;
        std::vector<char> seen(cap, 0);
        for (int p = 0; p < L; p++)
            for (int b = 0; b < B; b++) {
                const int i = sidx<LOG_L, B, ES>(p, b);
                if (i < 0 || (size_t)i >= cap || seen[i]) {
                    printf("FAIL es=%d L=2^%d B=%d: index %d of (p=%d, b=%d) out of range or repeated\n",
                           ES, LOG_L, B, i, p, b);
                    return false;
                }
                seen[i] = 1;
            }
        /* the stages: (radix, NS, reads, writes) as fft_line_regs runs them */
        struct St {
            int r, ns;
            bool from, to;
        };
        std::vector<St> st;
        const int r0 = SH::LR0 ? SH::R0 : 16;
        st.push_back({r0, 1, false, true});
        const int first_log = SH::LR0 ? SH::LR0 : SH::LE;
        for (int s = 1; s < SH::NSTAGE; s++)
            st.push_back({16, 1 << (first_log + SH::LE * (s - 1)), true, s != SH::NSTAGE - 1});
        Count c;
        std::vector<long> addr(32);
        for (const St &g : st) {
            for (int w0 = 0; w0 < NT; w0 += 32) {
                if (g.from)
                    for (int q = 0; q < E; q++) {
                        for (int t = 0; t < 32; t++) {
                            const int j = (w0 + t) / B, b = (w0 + t) % B;
                            addr[t] = (long)sidx<LOG_L, B, ES>(j + q * TPL, b) * ES;
                        }
                        add_request(addr, ES, c);
                    }
                if (g.to)
                    for (int u = 0; u < E / g.r; u++)
                        for (int r = 0; r < g.r; r++) {
                            for (int t = 0; t < 32; t++) {
                                const int j = (w0 + t) / B, b = (w0 + t) % B;
                                const int jj = j + u * TPL, k = jj & (g.ns - 1);
                                const int o = (jj / g.ns) * g.ns * g.r + k;
                                addr[t] = (long)sidx<LOG_L, B, ES>(o + r * g.ns, b) * ES;
                            }
                            add_request(addr, ES, c);
                        }
            }
        }
        bool ok = c.waves == c.ideal;
        printf("%s es=%d L=2^%d B=%d: %ld wavefronts, minimum %ld\n", ok ? "ok  " : "FAIL", ES, LOG_L, B,
               c.waves, c.ideal);
        /* tiles of B >= 8 whole lines staged by bulk copies: thread (j, b)
         * reads element j + q * TPL of line b's slot.  Slots start on 16-byte
         * boundaries, so 16 lines of 8-byte elements read at one index cannot
         * all fall in distinct bank pairs: two wavefronts per phase there */
        if (B >= 8 && (size_t)L * ES >= 512) {
            Count cb;
            const long slot = (long)bulk_slot_bytes(LOG_L, ES);
            for (int w0 = 0; w0 < NT; w0 += 32)
                for (int q = 0; q < E; q++) {
                    for (int t = 0; t < 32; t++) {
                        const int j = (w0 + t) / B, b = (w0 + t) % B;
                        addr[t] = b * slot + (long)(j + q * TPL) * ES;
                    }
                    add_request(addr, ES, cb);
                }
            const long allowed = (ES == 8 && B >= 16) ? 2 * cb.ideal : cb.ideal;
            const bool okb = cb.waves <= allowed;
            printf("%s es=%d L=2^%d B=%d staged tile reads: %ld wavefronts, minimum %ld%s\n", okb ? "ok  " : "FAIL",
                   ES, LOG_L, B, cb.waves, cb.ideal, allowed > cb.ideal ? " (two per phase allowed)" : "");
            ok = ok && okb;
        }
        return ok;
    }
}

template <int ES, int LOG_L, int... LB>
static bool row(std::integer_sequence<int, LB...>)
{
    constexpr int maxp = ES == 8 ? 14 : 13;
    bool ok = true;
    ((ok = ((LOG_L + LB <= maxp) ? check<ES, LOG_L, (1 << LB)>() : true) && ok), ...);
    return ok;
}

template <int ES, int... LL>
static bool all(std::integer_sequence<int, LL...>)
{
    bool ok = true;
    ((ok = row<ES, LL + 5>(std::make_integer_sequence<int, 6>{}) && ok), ...);
    return ok;
}

int main()
{
    bool ok = all<8>(std::make_integer_sequence<int, 9>{});
    ok = all<16>(std::make_integer_sequence<int, 9>{}) && ok;
    return ok ? 0 : 1;
}
