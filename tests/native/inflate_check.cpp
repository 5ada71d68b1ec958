// Host check of the DEFLATE decoder and CRC-32 of fame_gb300/csrc/inflate.h
// against zlib: streams from every compression level and strategy (stored,
// fixed-code, dynamic-code, Huffman-only and run-length blocks) over random
// bytes, FASTQ-like text and long runs, sizes 0 .. 64 KiB; then truncated and
// corrupted streams, which must give an error or a correct result and never
// write past the output.  Also the closed forms of the length and distance
// tables against RFC 1951's table, and the BGZF member header parser.  Prints "ok <streams>" or the first failure.
#include <zlib.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "inflate.h"

using namespace fame;

static std::vector<uint8_t> deflate_raw(const std::vector<uint8_t>& in, int level, int strategy)
{
    z_stream z{};
    if (deflateInit2(&z, level, Z_DEFLATED, -15, 8, strategy) != Z_OK) exit(2);
    std::vector<uint8_t> out(deflateBound(&z, in.size()) + 64);
    z.next_in = (Bytef*)in.data();
    z.avail_in = (uInt)in.size();
    z.next_out = out.data();
    z.avail_out = (uInt)out.size();
    if (deflate(&z, Z_FINISH) != Z_STREAM_END) exit(3);
    out.resize(z.total_out);
    deflateEnd(&z);
    return out;
}

static std::vector<uint8_t> make_data(std::mt19937_64& rng, int kind, size_t n)
{
    std::vector<uint8_t> d(n);
    if (kind == 0) {
        for (auto& c : d) c = (uint8_t)rng();
    } else if (kind == 1) {   // FASTQ-like records
        std::string s;
        while (s.size() < n) {
            const int L = 36 + (int)(rng() % 115);
            s += "@read" + std::to_string(rng() % 1000000) + "\n";
            for (int i = 0; i < L; ++i) s += "ACGT"[rng() % 4];
            s += "\n+\n";
            for (int i = 0; i < L; ++i) s += (char)('5' + rng() % 10);
            s += "\n";
        }
        if (n) std::memcpy(d.data(), s.data(), n);
    } else {   // runs
        size_t i = 0;
        while (i < n) {
            const size_t r = std::min<size_t>(n - i, 1 + rng() % 3000);
            std::memset(d.data() + i, (int)(rng() % 4), r);
            i += r;
        }
    }
    return d;
}

int main()
{
    // closed forms of RFC 1951's length and distance tables
    const uint32_t lb[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115,
                             131, 163, 195, 227, 258};
    const uint32_t le[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    const uint32_t db[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537,
                             2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    for (uint32_t i = 0; i < 29; ++i)
        if (infl_len_base(i) != lb[i] || infl_len_extra(i) != le[i]) { printf("length table %u\n", i); return 1; }
    for (uint32_t i = 0; i < 30; ++i)
        if (infl_dist_base(i) != db[i] || infl_dist_extra(i) != (i < 4 ? 0 : (i - 2) / 2)) { printf("distance table %u\n", i); return 1; }
    uint32_t tab[256];
    crc32_table(tab);
    static InflScratch sc;
    std::mt19937_64 rng(777);
    const int levels[] = {0, 1, 6, 9};
    const int strategies[] = {Z_DEFAULT_STRATEGY, Z_FILTERED, Z_HUFFMAN_ONLY, Z_RLE, Z_FIXED};
    const size_t sizes[] = {0, 1, 2, 100, 4096, 65535, 65536};
    long streams = 0;
    for (int kind = 0; kind < 3; ++kind)
        for (size_t n : sizes)
            for (int lv : levels)
                for (int st : strategies) {
                    const std::vector<uint8_t> data = make_data(rng, kind, n);
                    const std::vector<uint8_t> c = deflate_raw(data, lv, st);
                    std::vector<uint8_t> out(n + 16, 0xAB);
                    uint32_t got = 0;
                    const int r = infl_raw(c.data(), (uint32_t)c.size(), out.data(), (uint32_t)n, &got, sc);
                    if (r != INFL_OK || got != n || (n && std::memcmp(out.data(), data.data(), n) != 0)) {
                        printf("stream kind %d size %zu level %d strategy %d: code %d, %u bytes\n", kind, n, lv, st, r, got);
                        return 1;
                    }
                    for (size_t i = n; i < n + 16; ++i)
                        if (out[i] != 0xAB) { printf("wrote past the output\n"); return 1; }
                    if (crc32_of(tab, data.data(), (uint32_t)n) != (uint32_t)crc32(0L, data.data(), (uInt)n)) {
                        printf("crc kind %d size %zu\n", kind, n);
                        return 1;
                    }
                    ++streams;
                    // a smaller output must be refused, not overrun
                    if (n > 0) {
                        std::vector<uint8_t> small(n - 1 + 16, 0xCD);
                        const int r2 = infl_raw(c.data(), (uint32_t)c.size(), small.data(), (uint32_t)(n - 1), &got, sc);
                        if (r2 == INFL_OK) { printf("short output accepted\n"); return 1; }
                        for (size_t i = n - 1; i < small.size(); ++i)
                            if (small[i] != 0xCD) { printf("wrote past a short output\n"); return 1; }
                    }
                    // truncations and flipped bytes: an error or the right bytes, within bounds
                    for (int t = 0; t < 12 && !c.empty(); ++t) {
                        std::vector<uint8_t> bad = c;
                        if (t < 4) bad.resize(rng() % c.size());
                        else bad[rng() % bad.size()] ^= (uint8_t)(1u + rng() % 255);
                        std::vector<uint8_t> o2(n + 16, 0xEF);
                        const int r3 = infl_raw(bad.data(), (uint32_t)bad.size(), o2.data(), (uint32_t)n, &got, sc);
                        for (size_t i = n; i < n + 16; ++i)
                            if (o2[i] != 0xEF) { printf("corrupt stream wrote past the output\n"); return 1; }
                        if (r3 == INFL_OK && got > n) { printf("corrupt stream: size\n"); return 1; }
                    }
                }
    // BGZF member parsing: sizes from the header's BC subfield and the trailer
    {
        const std::vector<uint8_t> data = make_data(rng, 1, 5000);
        const std::vector<uint8_t> c = deflate_raw(data, 6, Z_DEFAULT_STRATEGY);
        std::vector<uint8_t> m = {31, 139, 8, 4, 0, 0, 0, 0, 0, 255, 6, 0, 'B', 'C', 2, 0, 0, 0};
        m.insert(m.end(), c.begin(), c.end());
        const uint32_t cr = (uint32_t)crc32(0L, data.data(), (uInt)data.size()), is = (uint32_t)data.size();
        for (int k = 0; k < 4; ++k) m.push_back((uint8_t)(cr >> (8 * k)));
        for (int k = 0; k < 4; ++k) m.push_back((uint8_t)(is >> (8 * k)));
        const uint32_t bsize = (uint32_t)m.size() - 1;
        m[16] = (uint8_t)bsize;
        m[17] = (uint8_t)(bsize >> 8);
        uint32_t cd, cl, crc, isz;
        if (bgzf_member(m.data(), m.size(), &cd, &cl, &crc, &isz) != m.size() || cd != 18 || cl != c.size() ||
            crc != cr || isz != is) { printf("bgzf member fields\n"); return 1; }
        std::vector<uint8_t> out(is);
        uint32_t got;
        if (infl_raw(m.data() + cd, cl, out.data(), isz, &got, sc) != INFL_OK || got != is || out != data ||
            crc32_of(tab, out.data(), got) != crc) { printf("bgzf member inflate\n"); return 1; }
        if (bgzf_member(m.data(), m.size() - 1, &cd, &cl, &crc, &isz) != 0) { printf("incomplete member accepted\n"); return 1; }
        std::vector<uint8_t> plain = m;
        plain[3] = 0;   // no FEXTRA: plain gzip
        if (bgzf_member(plain.data(), plain.size(), &cd, &cl, &crc, &isz) != 0) { printf("plain gzip accepted\n"); return 1; }
        std::vector<uint8_t> other = m;
        other[12] = 'X';   // another subfield
        if (bgzf_member(other.data(), other.size(), &cd, &cl, &crc, &isz) != 0) { printf("foreign subfield accepted\n"); return 1; }
    }
    printf("ok %ld\n", streams);
    return 0;
}
