// Host check of the bit-vector scan (fame_gb300/csrc/editscan.h): at every
// text position its answer must equal the 7-layer ShiftAnd<6> automaton's
// (ShiftAnd.h:276-341), restated below in its direct form.  Texts carry N
// runs (both reset), patterns carry N bases and read T's (which also accept
// a text C).  Prints "ok <cases> <positions>" or the first differing case.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "editscan.h"

using namespace fame;

struct ShiftAnd {
    int W = 0;
    uint32_t m = 0;
    std::vector<uint64_t> mask[4], acc, act[NERR + 1];

    void load(const std::string& p)
    {
        m = (uint32_t)p.size();
        W = (int)(m / 64 + 1);
        for (auto& v : mask) v.assign(W, 0);
        acc.assign(W, 0);
        for (auto& v : act) v.assign(W, 0);
        acc[m / 64] = 1ull << (m % 64);
        // bit j + 1 of mask[c]: read position j accepts text letter c; bit 0 always set
        for (int c = 0; c < 4; ++c) mask[c][0] = 1;
        for (uint32_t j = 0; j < m; ++j) {
            const uint32_t bit = j + 1;
            auto set = [&](int c) { mask[c][bit / 64] |= 1ull << (bit % 64); };
            switch (p[j]) {
                case 'A': set(0); break;
                case 'C': set(1); break;
                case 'G': set(2); break;
                case 'T': set(3); set(1); break;
                default: break;
            }
        }
    }
    void reset()
    {
        for (int i = 0; i <= (int)NERR; ++i) {
            for (int j = 0; j < W; ++j) act[i][j] = 0;
            act[i][0] = (1ull << (i + 1)) - 1;
        }
    }
    static uint64_t shl(const std::vector<uint64_t>& v, int j) { return (v[j] << 1) | (j ? v[j - 1] >> 63 : 0); }
    void letter(int b)
    {
        const std::vector<uint64_t>& mk = mask[b];
        for (int i = NERR; i > 0; --i)
            for (int j = W - 1; j >= 0; --j)
                act[i][j] = ((shl(act[i], j) | (j ? 0 : 1)) & mk[j]) | act[i - 1][j] | shl(act[i - 1], j);
        for (int j = W - 1; j >= 0; --j) act[0][j] = (shl(act[0], j) | (j ? 0 : 1)) & mk[j];
        for (int i = 1; i <= (int)NERR; ++i)
            for (int j = W - 1; j >= 0; --j) act[i][j] |= shl(act[i - 1], j);
    }
    int match() const
    {
        for (int i = 0; i <= (int)NERR; ++i)
            for (int j = 0; j < W; ++j)
                if (act[i][j] & acc[j]) return i;
        return -1;
    }
};

template <int W>
static bool run_case(const std::string& pat, int orient, const std::string& text, uint64_t& npos)
{
    // the scan's read position p is pat[p] (orient 0) or the complement of pat[len-1-p]
    std::string eff = pat;
    if (orient) {
        for (size_t p = 0; p < pat.size(); ++p) {
            const char c = pat[pat.size() - 1 - p];
            eff[p] = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : 'N';
        }
    }
    ShiftAnd sa;
    sa.load(eff);
    sa.reset();
    EditScan<W> es;
    es.load(pat.data(), (uint32_t)pat.size(), orient);
    es.reset();
    for (size_t t = 0; t < text.size(); ++t) {
        const char c = text[t];
        if (c == 'N') { sa.reset(); es.reset(); continue; }
        const int b = c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : 3;
        sa.letter(b);
        es.letter(b);
        ++npos;
        if (sa.match() != es.match()) {
            std::printf("DIFF m=%zu orient=%d t=%zu shiftand=%d editscan=%d\n", pat.size(), orient, t, sa.match(),
                        es.match());
            return false;
        }
    }
    return true;
}

int main(int argc, char** argv)
{
    const int cases = argc > 1 ? atoi(argv[1]) : 3000;
    std::mt19937_64 rng(777);
    const char* ACGT = "ACGT";
    uint64_t npos = 0;
    for (int cs = 0; cs < cases; ++cs) {
        // lengths over every width, weighted to the 64-bit word edges
        uint32_t m;
        switch (cs % 5) {
            case 0: m = 7 + (uint32_t)(rng() % 249); break;
            case 1: m = 60 + (uint32_t)(rng() % 9); break;
            case 2: m = 124 + (uint32_t)(rng() % 9); break;
            case 3: m = 188 + (uint32_t)(rng() % 9); break;
            default: m = 80 + (uint32_t)(rng() % 71); break;
        }
        if (m > 255) m = 255;
        std::string pat(m, 'A');
        for (auto& c : pat) {
            const uint64_t r = rng() % 100;
            c = r < 2 ? 'N' : ACGT[rng() & 3];
        }
        // text: mutated copies of the pattern (so matches occur at every error
        // count), random stretches and N runs
        std::string text;
        while (text.size() < 3 * m + 200) {
            const uint64_t r = rng() % 10;
            if (r < 5) {
                std::string s = pat;
                for (auto& c : s) if (c == 'N') c = ACGT[rng() & 3];
                const int edits = (int)(rng() % 9);
                for (int e = 0; e < edits && !s.empty(); ++e) {
                    const size_t pos = rng() % s.size();
                    const int kind = (int)(rng() % 3);
                    if (kind == 0) s[pos] = ACGT[rng() & 3];
                    else if (kind == 1) s.erase(pos, 1);
                    else s.insert(pos, 1, ACGT[rng() & 3]);
                }
                // read T's align to text C's under the bisulfite rule
                for (auto& c : s) if (c == 'T' && rng() % 4 == 0) c = 'C';
                text += s;
            } else if (r < 8) {
                for (int i = (int)(rng() % 40); i >= 0; --i) text.push_back(ACGT[rng() & 3]);
            } else {
                text.append(1 + rng() % 3, 'N');
            }
        }
        const int orient = (int)(rng() & 1);
        std::string pt = pat;
        if (orient) {
            // the scan complements the reversed read: feed the reverse complement's source
            std::string src(m, 'A');
            for (size_t p = 0; p < m; ++p) {
                const char c = pat[m - 1 - p];
                src[p] = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : 'N';
            }
            pt = src;
        }
        bool ok;
        switch (m / 64 + 1) {
            case 1: ok = run_case<1>(pt, orient, text, npos); break;
            case 2: ok = run_case<2>(pt, orient, text, npos); break;
            case 3: ok = run_case<3>(pt, orient, text, npos); break;
            default: ok = run_case<4>(pt, orient, text, npos); break;
        }
        if (!ok) return 1;
    }
    std::printf("ok %d %llu\n", cases, (unsigned long long)npos);
    return 0;
}
