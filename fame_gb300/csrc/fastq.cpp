// FASTQ chunk reader: parseChunk / parseChunkGZ (ReadQueue.cpp:218-373) for
// the GPU path.  A record is four lines and its sequence is the second; as in
// the reference nothing is validated.  The sequences of up to max_reads
// records are packed back to back with offsets, the layout the match calls
// take (the caller may pass page-locked buffers from fame_gpu_host_alloc).
//
// The file is read in 64 MB blocks of whole lines; threads count the lines of
// their part of a block, a prefix over those counts gives each part its first
// line number, each thread copies the sequence lines (number % 4 == 1) of its
// part, and the parts are concatenated in order.  A call stops at the record
// after its max_reads-th sequence, so the next call starts on a record.  Gzip
// input is inflated with zlib on the calling thread.
#include <zlib.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fame_gpu.h"

struct fame_fastq {
    FILE* f = nullptr;
    gzFile gz = nullptr;
    std::vector<char> buf;   // unread bytes start at pos
    size_t pos = 0, len = 0;
    bool eof = false;
    uint64_t line = 0;       // line number of buf[pos] (records start at multiples of 4)
    int threads = 1;
};

namespace {

constexpr size_t BLOCK = 64u << 20;

// Appends up to `want` more bytes of input after the unread ones.
bool fill(fame_fastq* q, size_t want)
{
    if (q->pos > 0) {
        std::memmove(q->buf.data(), q->buf.data() + q->pos, q->len - q->pos);
        q->len -= q->pos;
        q->pos = 0;
    }
    if (q->buf.size() < q->len + want) q->buf.resize(q->len + want);
    size_t got = 0;
    while (got < want && !q->eof) {
        long r;
        if (q->gz) {
            const int n = gzread(q->gz, q->buf.data() + q->len + got, (unsigned)std::min<size_t>(want - got, 1u << 30));
            if (n < 0) return false;
            r = n;
        } else {
            r = (long)std::fread(q->buf.data() + q->len + got, 1, want - got, q->f);
            if (r == 0 && std::ferror(q->f)) return false;
        }
        if (r == 0) q->eof = true;
        got += (size_t)r;
    }
    q->len += got;
    return true;
}

}  // namespace

extern "C" int fame_fastq_open(const char* path, int is_gz, int n_threads, fame_fastq** out)
{
    if (!path || !out) return FAME_ERR_ARG;
    *out = nullptr;
    fame_fastq* q = new (std::nothrow) fame_fastq();
    if (!q) return FAME_ERR_NOMEM;
    if (is_gz) q->gz = gzopen(path, "rb");
    else q->f = std::fopen(path, "rb");
    if (!q->f && !q->gz) {
        delete q;
        return FAME_ERR_IO;
    }
    q->threads = n_threads > 0 ? n_threads : (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    *out = q;
    return FAME_OK;
}

extern "C" int fame_fastq_read(fame_fastq* q, uint32_t max_reads, char* seqs, uint64_t seq_cap, uint64_t* offs,
                               uint32_t* n_out)
{
    if (!q || !seqs || !offs || !n_out) return FAME_ERR_ARG;
    *n_out = 0;
    offs[0] = 0;
    uint32_t n = 0;
    uint64_t used = 0;
    while (n < max_reads) {
        if (q->len - q->pos < BLOCK / 2 && !q->eof)
            if (!fill(q, BLOCK)) return FAME_ERR_IO;
        const char* base = q->buf.data() + q->pos;
        const size_t avail = q->len - q->pos;
        if (avail == 0) break;
        // the block: whole lines, or everything once the input has ended
        size_t end = avail;
        if (!q->eof) {
            const char* nl = (const char*)memrchr(base, '\n', avail);
            if (!nl) {
                if (!fill(q, BLOCK)) return FAME_ERR_IO;
                continue;
            }
            end = (size_t)(nl - base) + 1;
        }
        // parts cut at line starts; their line counts, in parallel
        const int T = std::max(1, std::min(q->threads, (int)(end >> 20) + 1));
        std::vector<size_t> cut(T + 1, 0);
        for (int t = 1; t < T; ++t) {
            const size_t c = std::max(cut[t - 1], end * (size_t)t / (size_t)T);
            const char* nl = c < end ? (const char*)std::memchr(base + c, '\n', end - c) : nullptr;
            cut[t] = nl ? (size_t)(nl - base) + 1 : end;
        }
        cut[T] = end;
        auto count_lines = [&](size_t a0, size_t a1) {
            uint64_t c = 0;
            for (const char* p = base + a0; p < base + a1;) {
                const char* nl = (const char*)std::memchr(p, '\n', (size_t)(base + a1 - p));
                ++c;
                if (!nl) break;
                p = nl + 1;
            }
            return c;
        };
        std::vector<uint64_t> lines(T, 0);
        {
            std::vector<std::thread> th;
            for (int t = 1; t < T; ++t) th.emplace_back([&, t] { lines[t] = count_lines(cut[t], cut[t + 1]); });
            lines[0] = count_lines(cut[0], cut[1]);
            for (auto& x : th) x.join();
        }
        // line number at each part's start; sequence lines are those with number % 4 == 1
        std::vector<uint64_t> first(T + 1, q->line);
        for (int t = 0; t < T; ++t) first[t + 1] = first[t] + lines[t];
        auto seqs_before = [](uint64_t l) { return (l + 2) / 4; };   // sequence lines with number < l
        const uint64_t s0 = seqs_before(q->line);
        const uint64_t room = max_reads - n;
        // the block ends the call when it holds room more sequences: stop at the start of the next record
        uint64_t stop_line = first[T];
        if (seqs_before(first[T]) - s0 > room) {
            // record k (0-based from here) starts at line 4 * (s0 + k); the next record after `room` sequences
            stop_line = 4 * (s0 + room);
        }
        // per part: its sequences below stop_line, copied to a per-part buffer, then concatenated
        std::vector<std::string> part(T);
        std::vector<std::vector<uint32_t>> plen(T);
        std::vector<size_t> pend(T, 0);
        {
            std::vector<std::thread> th;
            auto run = [&](int t) {
                uint64_t line = first[t];
                const char* p = base + cut[t];
                const char* pe = base + cut[t + 1];
                while (p < pe && line < stop_line) {
                    const char* nl = (const char*)std::memchr(p, '\n', (size_t)(pe - p));
                    const char* le = nl ? nl : pe;
                    if (line % 4 == 1) {
                        part[t].append(p, (size_t)(le - p));
                        plen[t].push_back((uint32_t)(le - p));
                    }
                    ++line;
                    p = nl ? nl + 1 : pe;
                }
                pend[t] = (size_t)(p - base);
            };
            for (int t = 1; t < T; ++t) th.emplace_back(run, t);
            run(0);
            for (auto& x : th) x.join();
        }
        size_t consumed = 0;
        for (int t = 0; t < T; ++t) {
            if (used + part[t].size() > seq_cap) return FAME_ERR_ARG;   // the caller's buffer is too small
            std::memcpy(seqs + used, part[t].data(), part[t].size());
            for (uint32_t l : plen[t]) {
                used += l;
                offs[++n] = used;
            }
            if (first[t] < stop_line) consumed = std::max(consumed, pend[t]);
        }
        q->pos += consumed;
        q->line = std::min(stop_line, first[T]);
        if (stop_line < first[T]) break;
        if (q->eof && q->pos >= q->len) break;
    }
    *n_out = n;
    return FAME_OK;
}

extern "C" int fame_fastq_close(fame_fastq* q)
{
    if (!q) return FAME_ERR_ARG;
    if (q->f) std::fclose(q->f);
    if (q->gz) gzclose(q->gz);
    delete q;
    return FAME_OK;
}
