// Report writers: printMethylationLevels (ReadQueue.cpp:1860-1893) and the
// single-cell matrix of printSCMethylationLevels (ReadQueue.cpp:1894-1921,
// header from the single-cell ReadQueue constructor), byte-identical to the
// reference's std::ofstream output.  CpGs are formatted in blocks by several
// host threads and written in order.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fame_gpu.h"

namespace {

inline void put_uint(std::string& out, uint64_t v)
{
    char buf[24];
    int n = 0;
    do {
        buf[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (n) out.push_back(buf[--n]);
}

const char* chrom_name(const fame_index_view* v, uint32_t c)
{
    return (v->chrom_name && c < v->n_chrom && v->chrom_name[c]) ? v->chrom_name[c] : "";
}

// Formats items [0, n) with fmt(i, out) on up to n_threads threads, in blocks,
// and writes the blocks to f in order.
template <class Fmt>
bool write_blocks(FILE* f, uint64_t n, int n_threads, Fmt fmt)
{
    const uint64_t block = 1 << 16;
    const uint64_t nblocks = (n + block - 1) / block;
    unsigned nt = n_threads > 0 ? (unsigned)n_threads : std::max(1u, std::thread::hardware_concurrency());
    nt = (unsigned)std::min<uint64_t>(nt, std::max<uint64_t>(1, nblocks));
    for (uint64_t b0 = 0; b0 < nblocks; b0 += nt) {
        const uint64_t b1 = std::min<uint64_t>(nblocks, b0 + nt);
        std::vector<std::string> bufs(b1 - b0);
        std::vector<std::thread> th;
        for (uint64_t b = b0; b < b1; ++b)
            th.emplace_back([&, b] {
                std::string& out = bufs[b - b0];
                out.reserve(block * 40);
                const uint64_t e = std::min<uint64_t>(n, (b + 1) * block);
                for (uint64_t i = b * block; i < e; ++i) fmt(i, out);
            });
        for (auto& t : th) t.join();
        for (auto& s : bufs)
            if (!s.empty() && fwrite(s.data(), 1, s.size(), f) != s.size()) return false;
    }
    return true;
}

}  // namespace

extern "C" int fame_report_cpg(const fame_index_view* v, const uint16_t* meth, const char* path, int n_threads)
{
    if (!v || !path || (v->n_cpg && (!meth || !v->cpg))) return FAME_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return FAME_ERR_IO;
    const uint32_t rl = v->readlen;
    const bool ok = write_blocks(f, v->n_cpg, n_threads, [&](uint64_t i, std::string& out) {
        out += chrom_name(v, v->cpg[i].chrom);
        out.push_back('\t');
        put_uint(out, (uint32_t)(v->cpg[i].pos + rl - 2));   // unsigned arithmetic of the reference
        for (int k = 0; k < 4; ++k) {
            out.push_back('\t');
            put_uint(out, meth[4 * i + k]);
        }
        out.push_back('\n');
    });
    return (std::fclose(f) == 0 && ok) ? FAME_OK : FAME_ERR_IO;
}

extern "C" int fame_report_sc_header(const fame_index_view* v, const char* path)
{
    if (!v || !path || (v->n_cpg && !v->cpg)) return FAME_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return FAME_ERR_IO;
    std::string out = "\nSC_ID\tCount_Type\t";
    for (uint64_t i = 0; i < v->n_cpg; ++i) {
        out += chrom_name(v, v->cpg[i].chrom);
        out.push_back('\t');
    }
    out += "\nSC_ID\tCount_Type\t";
    for (uint64_t i = 0; i < v->n_cpg; ++i) {
        put_uint(out, (uint32_t)(v->cpg[i].pos + v->readlen - 2));
        out.push_back('\t');
    }
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    return (std::fclose(f) == 0 && ok) ? FAME_OK : FAME_ERR_IO;
}

extern "C" int fame_report_sc_rows(const fame_index_view* v, const char* sc_id, const uint16_t* meth, const char* path,
                                   int n_threads)
{
    if (!v || !sc_id || !path || (v->n_cpg && !meth)) return FAME_ERR_ARG;
    FILE* f = std::fopen(path, "ab");
    if (!f) return FAME_ERR_IO;
    // the fourth row carries the label "unmethFwd" as in the reference (ReadQueue.cpp:1915)
    static const char* labels[4] = {"methFwd", "unmethFwd", "methRev", "unmethFwd"};
    bool ok = true;
    for (int k = 0; k < 4 && ok; ++k) {
        std::string head = "\n";
        head += sc_id;
        head.push_back('\t');
        head += labels[k];
        head.push_back('\t');
        ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
        if (ok)
            ok = write_blocks(f, v->n_cpg, n_threads, [&](uint64_t i, std::string& out) {
                put_uint(out, meth[4 * i + k]);
                out.push_back('\t');
            });
    }
    return (std::fclose(f) == 0 && ok) ? FAME_OK : FAME_ERR_IO;
}
