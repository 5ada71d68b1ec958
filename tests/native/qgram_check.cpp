// Host check of the q-gram pre-filter (fame_gb300/csrc/qgram.h): its spans
// must equal those of the direct scan-order formulation below, which walks
// the window text in scan order one base at a time.  Prints "ok <cases>" or
// the first differing case.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <utility>
#include <vector>

#include "qgram.h"

using namespace fame;

static int scan_order_spans(const std::vector<uint32_t>& pack, const std::vector<uint32_t>& nm, uint64_t G0,
                            uint64_t G1, int fwd, uint32_t m, uint32_t q, const uint32_t* pkey, uint32_t pvalid,
                            const uint32_t* pstart, std::vector<std::pair<int, int>>& out, int cap)
{
    const int32_t len = (int32_t)(G1 - G0);
    const uint32_t qmask = q >= 16 ? 0xffffffffu : ((1u << (2 * q)) - 1);
    uint32_t key = 0, valid = 0;
    int n = 0;
    for (int32_t u = 0; u < len; ++u) {
        const uint64_t g = fwd ? G0 + (uint64_t)u : G1 - 1 - (uint64_t)u;
        if ((nm[g >> 5] >> (g & 31)) & 1u) { valid = 0; continue; }
        int b = (int)((pack[g >> 4] >> (2 * (g & 15))) & 3u);
        if (!fwd) b = 3 - b;
        const uint32_t sym = b == 0 ? 0u : (b == 2 ? 1u : 2u);
        key = ((key << 2) | sym) & qmask;
        if (++valid < q) continue;
        for (int k = 0; k < QG_PIECES; ++k) {
            if (!((pvalid >> k) & 1u) || key != pkey[k]) continue;
            const int32_t x = u - (int32_t)q + 1;
            const int32_t end0 = x - 1 + (int32_t)(m - pstart[k]);
            int32_t a = end0 - (int32_t)NERR, bb = end0 + (int32_t)NERR;
            if (bb < 0 || a > len - 1) continue;
            a = std::max(a, 0);
            bb = std::min(bb, len - 1);
            if (n >= cap) return -1;
            out.push_back({a, bb});
            ++n;
        }
    }
    return n;
}

int main(int argc, char** argv)
{
    const int cases = argc > 1 ? atoi(argv[1]) : 20000;
    std::mt19937_64 rng(12345);
    const uint64_t GL = 1 << 16;
    std::vector<uint32_t> pack(GL / 16 + 1), nm(GL / 32 + 1);
    std::vector<uint8_t> base(GL);
    for (uint64_t g = 0; g < GL; ++g) {
        // low-complexity stretches make repeated q-grams (and CAP overflows) common
        base[g] = (g / 512) % 7 == 3 ? (uint8_t)((g / 3) % 2 * 2) : (uint8_t)(rng() & 3);
        pack[g >> 4] |= (uint32_t)base[g] << (2 * (g & 15));
        if (rng() % 400 == 0 || ((g / 4096) % 5 == 2 && (g % 4096) < 40)) nm[g >> 5] |= 1u << (g & 31);
    }
    int total_spans = 0, overflows = 0;
    for (int c = 0; c < cases; ++c) {
        const int fwd = (int)(rng() & 1);
        const uint32_t len = rng() % 5 == 0 ? (uint32_t)(rng() % 40) : 1500 + (uint32_t)(rng() % 600);
        const uint64_t G0 = rng() % (GL - len - 1);
        const uint64_t G1 = G0 + len;
        const uint32_t m = 32 + (uint32_t)(rng() % 224);
        const uint32_t q = std::min<uint32_t>(16, m / 7);
        uint32_t pkey[QG_PIECES], pstart[QG_PIECES], pvalid = 0;
        for (int k = 0; k < QG_PIECES; ++k) {
            pstart[k] = (uint32_t)((k * m) / 7);
            if (rng() % 8 != 0) pvalid |= 1u << k;
            if (len > q && rng() % 3 != 0) {
                // the scan-order key of a text q-gram of this window
                const uint32_t x = (uint32_t)(rng() % (len - q + 1));
                uint32_t kk = 0;
                for (uint32_t i = 0; i < q; ++i) {
                    const uint64_t g = fwd ? G0 + x + i : G1 - 1 - (x + i);
                    int b = base[g];
                    if (!fwd) b = 3 - b;
                    kk = (kk << 2) | (b == 0 ? 0u : (b == 2 ? 1u : 2u));
                }
                pkey[k] = kk;
            } else {
                pkey[k] = (uint32_t)rng() & (q >= 16 ? 0xffffffffu : ((1u << (2 * q)) - 1));
            }
        }
        std::vector<std::pair<int, int>> want;
        const int nw = scan_order_spans(pack, nm, G0, G1, fwd, m, q, pkey, pvalid, pstart, want, 32);
        int32_t lo[32], hi[32];
        const int ng = qgram_spans<32>(pack.data(), nm.data(), G0, G1, fwd, m, q, pkey, pvalid, pstart, lo, hi);
        std::vector<std::pair<int, int>> got;
        for (int i = 0; i < ng; ++i) got.push_back({lo[i], hi[i]});
        std::sort(want.begin(), want.end());
        std::sort(got.begin(), got.end());
        if (nw != ng || (nw >= 0 && want != got)) {
            printf("mismatch case %d fwd %d G0 %llu len %u m %u q %u: scan-order %d spans, filter %d\n", c, fwd,
                   (unsigned long long)G0, len, m, q, nw, ng);
            return 1;
        }
        if (nw < 0) ++overflows;
        else total_spans += nw;
    }
    printf("ok %d cases, %d spans, %d overflows\n", cases, total_spans, overflows);
    return 0;
}
