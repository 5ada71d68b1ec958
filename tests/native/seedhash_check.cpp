// Host check of the prefix form of the spaced-seed hash (fame_gb300/csrc/seedhash.h):
// for random reads of every length up to 255 (ACGT, lower case, N and other
// bytes), the table index of every k-mer must equal the direct form's.
// Prints "ok <kmers>" or the first differing k-mer.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "seedhash.h"

using namespace fame;

int main(int argc, char** argv)
{
    const int cases = argc > 1 ? atoi(argv[1]) : 20000;
    std::mt19937_64 rng(4242);
    const char* alpha = "ACGTACGTACGTacgtN\x01\x03\x04\x07Z";
    uint64_t nk = 0;
    for (int cs = 0; cs < cases; ++cs) {
        const uint32_t len = KMERLEN + (uint32_t)(rng() % (256 - KMERLEN));
        std::vector<uint8_t> seq(len);
        for (auto& c : seq) c = (uint8_t)alpha[rng() % 22];
        std::vector<uint64_t> P(len + 1, 0);
        for (uint32_t j = 0; j < len; ++j) P[j + 1] = P[j] ^ sh_u(seq[j], j);
        for (uint32_t p = 0; p + KMERLEN <= len; ++p) {
            const uint32_t d = (uint32_t)(sh_direct(seq.data(), p) & HTAB_MASK);
            const uint32_t f = sh_prefix_hash([&](uint32_t j) { return P[j]; }, p, HTAB_MASK);
            ++nk;
            if (d != f) {
                std::printf("DIFF len=%u p=%u direct=%08x prefix=%08x\n", len, p, d, f);
                return 1;
            }
        }
    }
    std::printf("ok %llu\n", (unsigned long long)nk);
    return 0;
}
