// FASTQ chunk reader: parseChunk / parseChunkGZ (ReadQueue.cpp:218-373) for
// the GPU path.  A record is four lines and its sequence is the second; as in
// the reference nothing is validated.  The sequences of up to max_reads
// records are packed back to back with offsets, the layout the match calls
// take (the caller may pass page-locked buffers from fame_gpu_host_alloc).
//
// Input: a regular uncompressed file is mapped and parsed in place (no copy
// out of the page cache); gzip input and pipes are read into a buffer (gzip
// inflated by zlib on the calling thread, or, for BGZF input opened with a
// device, member by member on the GPU: the compressed bytes are read in 64 MiB
// pieces, the complete members found from their headers, and each refill
// inflates enough of them in one launch).  A call parses a region of whole
// lines sized from the bytes per record seen so far, in two parallel passes
// over parts cut at line starts: the first counts each part's lines and, for
// each of the four possible line phases, its sequence lines and their bytes;
// a prefix over the parts gives every part its first line number, hence its
// phase, its first record and its first output byte; the second pass copies
// the part's sequence lines straight to their place in the caller's buffer
// and writes their offsets.  A call stops at the record after its
// max_reads-th sequence, so the next call starts on a record.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>
#include <zlib.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/fame_gpu.h"
#include "bgzf.h"
#include "inflate.h"

namespace {

// Workers 1..T-1 run job(t) for each dispatch; the caller runs job(0).
class Pool {
public:
    explicit Pool(int T) : T_(T)
    {
        for (int t = 1; t < T; ++t) th_.emplace_back([this, t] { loop(t); });
    }
    ~Pool()
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& x : th_) x.join();
    }
    int size() const { return T_; }
    void run(const std::function<void(int)>& job)
    {
        if (T_ == 1) {
            job(0);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = &job;
            remaining_ = T_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        job(0);
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [this] { return remaining_ == 0; });
        job_ = nullptr;
    }

private:
    void loop(int t)
    {
        uint64_t seen = 0;
        for (;;) {
            const std::function<void(int)>* job;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                job = job_;
            }
            (*job)(t);
            std::lock_guard<std::mutex> lk(m_);
            if (--remaining_ == 0) done_.notify_one();
        }
    }
    int T_;
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    const std::function<void(int)>* job_ = nullptr;
    uint64_t gen_ = 0;
    int remaining_ = 0;
    bool stop_ = false;
};

constexpr size_t BLOCK = 64u << 20;     // first region, and the buffer's refill size
constexpr size_t CREAD = 64u << 20;     // compressed bytes read at a time (BGZF input)
constexpr size_t MIN_PART = 1u << 16;   // smallest part worth a thread

}  // namespace

struct fame_fastq {
    // a regular uncompressed file: mapped
    const char* map = nullptr;
    size_t map_len = 0;
    size_t dropped = 0;       // mapped pages before this offset are released
    // otherwise: FILE / gzip stream read into buf
    FILE* f = nullptr;
    gzFile gz = nullptr;
    // BGZF input inflated on the GPU: compressed bytes [cpos, clen) of cbuf unread
    FILE* cf = nullptr;
    fame::BgzfGpu* bgzf = nullptr;
    std::vector<uint8_t> cbuf;
    size_t cpos = 0, clen = 0;
    bool ceof = false;
    std::vector<char> buf;
    bool eof = false;
    size_t pos = 0, len = 0;  // unread bytes: [pos, len) of the mapping or of buf
    uint64_t line = 0;        // line number at pos (records start at multiples of 4)
    double bytes_per_seq = 0; // input bytes per record so far (region sizing)
    Pool* pool = nullptr;
};

namespace {

// More compressed input after the unread bytes; false on a read error.
bool read_compressed(fame_fastq* q, size_t* scan)
{
    if (q->cpos > 0) {   // the unread compressed bytes to the front
        std::memmove(q->cbuf.data(), q->cbuf.data() + q->cpos, q->clen - q->cpos);
        *scan -= q->cpos;
        q->clen -= q->cpos;
        q->cpos = 0;
    }
    if (q->cbuf.size() < q->clen + CREAD) q->cbuf.resize(q->clen + CREAD);
    const size_t r = std::fread(q->cbuf.data() + q->clen, 1, CREAD, q->cf);
    if (r == 0) {
        if (std::ferror(q->cf)) return false;
        q->ceof = true;
    }
    q->clen += r;
    return true;
}

// BGZF input: the complete members giving at least `want` bytes (or all that
// are left) inflated on the GPU after the unread bytes.  False on a read
// error, a malformed or truncated member, or a member that is not BGZF.
bool fill_bgzf(fame_fastq* q, size_t want)
{
    std::vector<fame::BgzfMember> ms;
    uint64_t out_total = 0;
    size_t scan = q->cpos;
    for (;;) {
        while (out_total < want) {
            uint32_t cd, cl, crc, isz;
            const uint32_t tot = fame::bgzf_member(q->cbuf.data() + scan, q->clen - scan, &cd, &cl, &crc, &isz);
            if (!tot) break;
            ms.push_back(fame::BgzfMember{(uint64_t)(scan - q->cpos) + cd, cl, crc, out_total, isz, 0});
            out_total += isz;
            scan += tot;
        }
        if (out_total >= want || q->ceof) break;
        if (!read_compressed(q, &scan)) return false;
    }
    if (q->ceof && out_total < want && scan < q->clen) return false;   // bytes left that are no complete member
    if (q->buf.size() < q->len + out_total) q->buf.resize(q->len + out_total);
    if (!ms.empty() && fame::bgzf_gpu_inflate(q->bgzf, q->cbuf.data() + q->cpos, scan - q->cpos, ms.data(),
                                              (uint32_t)ms.size(), (uint8_t*)q->buf.data() + q->len, out_total) != FAME_OK)
        return false;
    q->len += out_total;
    q->cpos = scan;
    if (q->ceof && q->cpos == q->clen) q->eof = true;
    return true;
}

// Appends up to `want` more bytes of buffered input after the unread ones.
bool fill(fame_fastq* q, size_t want)
{
    if (q->pos > 0) {
        std::memmove(q->buf.data(), q->buf.data() + q->pos, q->len - q->pos);
        q->len -= q->pos;
        q->pos = 0;
    }
    if (q->bgzf) return fill_bgzf(q, want);
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

const char* data(const fame_fastq* q) { return q->map ? q->map : q->buf.data(); }
bool at_end(const fame_fastq* q) { return q->map ? true : q->eof; }

// Per part: line count and, for local phase k (line index % 4 == k), the
// number of such lines and their bytes without the newline.
struct PartCount {
    uint64_t lines = 0;
    uint64_t n[4] = {0, 0, 0, 0};
    uint64_t bytes[4] = {0, 0, 0, 0};
};

uint64_t seqs_before(uint64_t l) { return (l + 2) / 4; }   // sequence lines (number % 4 == 1) below line l

// One region [base, base + end) of whole lines (the last may lack its newline
// at the end of the input): appends its sequences below the stop line to
// seqs / offs.  Returns FAME_OK or FAME_ERR_ARG when seq_cap is too small.
int parse_region(fame_fastq* q, const char* base, size_t end, uint32_t room, char* seqs, uint64_t seq_cap,
                 uint64_t* offs, uint32_t* n, uint64_t* used, size_t* consumed, uint64_t* lines_done)
{
    const int T = std::max(1, std::min(q->pool->size(), (int)(end / MIN_PART) + 1));
    std::vector<size_t> cut(T + 1, 0);
    for (int t = 1; t < T; ++t) {
        const size_t c = std::max(cut[t - 1], end * (size_t)t / (size_t)T);
        const char* nl = c < end ? (const char*)std::memchr(base + c, '\n', end - c) : nullptr;
        cut[t] = nl ? (size_t)(nl - base) + 1 : end;
    }
    cut[T] = end;
    std::vector<PartCount> pc(T);
    q->pool->run([&](int t) {
        if (t >= T) return;
        PartCount c;
        const char* p = base + cut[t];
        const char* pe = base + cut[t + 1];
        while (p < pe) {
            const char* nl = (const char*)std::memchr(p, '\n', (size_t)(pe - p));
            const char* le = nl ? nl : pe;
            const int k = (int)(c.lines & 3);
            ++c.n[k];
            c.bytes[k] += (uint64_t)(le - p);
            ++c.lines;
            p = nl ? nl + 1 : pe;
        }
        pc[t] = c;
    });
    // each part's first line, record and output byte
    std::vector<uint64_t> first(T + 1), rec(T), byte(T);
    first[0] = q->line;
    uint64_t r = *n, b = *used;
    for (int t = 0; t < T; ++t) {
        first[t + 1] = first[t] + pc[t].lines;
        const int k = (int)((1 - first[t]) & 3);
        rec[t] = r;
        byte[t] = b;
        r += pc[t].n[k];
        b += pc[t].bytes[k];
    }
    const uint64_t s0 = seqs_before(q->line);
    uint64_t stop_line = first[T];
    if (seqs_before(first[T]) - s0 > room) stop_line = 4 * (s0 + room);   // the record after `room` sequences
    std::vector<size_t> stop_at(T, SIZE_MAX);
    std::atomic<int> overflow{0};
    q->pool->run([&](int t) {
        if (t >= T || first[t] > stop_line) return;
        uint64_t line = first[t], ob = byte[t], orec = rec[t];
        const char* p = base + cut[t];
        const char* pe = base + cut[t + 1];
        while (p < pe) {
            if (line == stop_line) {
                stop_at[t] = (size_t)(p - base);
                return;
            }
            const char* nl = (const char*)std::memchr(p, '\n', (size_t)(pe - p));
            const char* le = nl ? nl : pe;
            if ((line & 3) == 1) {
                const uint64_t len = (uint64_t)(le - p);
                if (ob + len > seq_cap) {
                    overflow.store(1, std::memory_order_relaxed);
                    return;
                }
                std::memcpy(seqs + ob, p, len);
                ob += len;
                offs[++orec] = ob;
            }
            ++line;
            p = nl ? nl + 1 : pe;
        }
    });
    if (overflow.load()) return FAME_ERR_ARG;   // the caller's buffer is too small
    size_t stop_byte = end;
    for (int t = 0; t < T; ++t)
        if (stop_at[t] != SIZE_MAX) { stop_byte = stop_at[t]; break; }
    const uint64_t got = seqs_before(stop_line) - s0;
    *n += (uint32_t)got;
    *used = got ? offs[*n] : *used;
    *consumed = stop_line < first[T] ? stop_byte : end;
    *lines_done = stop_line - q->line;
    return FAME_OK;
}

}  // namespace

extern "C" int fame_fastq_open(const char* path, int is_gz, int n_threads, fame_fastq** out)
{
    return fame_fastq_open_dev(path, is_gz, n_threads, -1, out);
}

extern "C" int fame_fastq_open_dev(const char* path, int is_gz, int n_threads, int device, fame_fastq** out)
{
    if (!path || !out) return FAME_ERR_ARG;
    *out = nullptr;
    fame_fastq* q = new (std::nothrow) fame_fastq();
    if (!q) return FAME_ERR_NOMEM;
    if (is_gz && device >= 0) {
        // BGZF when the first member is complete and BGZF's (the first 64 MiB read either way)
        q->cf = std::fopen(path, "rb");
        if (q->cf) {
            size_t scan = 0;
            uint32_t cd, cl, crc, isz;
            if (!read_compressed(q, &scan) || !fame::bgzf_member(q->cbuf.data(), q->clen, &cd, &cl, &crc, &isz)) {
                std::fclose(q->cf);
                q->cf = nullptr;
                q->cbuf.clear();
                q->clen = 0;
                q->ceof = false;
            } else if (!(q->bgzf = fame::bgzf_gpu_open(device))) {
                fame_fastq_close(q);
                return FAME_ERR_CUDA;
            }
        }
    }
    if (q->bgzf) {
        // read through fill_bgzf
    } else if (is_gz) {
        q->gz = gzopen(path, "rb");
        if (q->gz) gzbuffer(q->gz, 1u << 20);
    } else {
        const int fd = ::open(path, O_RDONLY);
        struct stat st;
        if (fd >= 0 && ::fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
            void* m = ::mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
            if (m != MAP_FAILED) {
                ::madvise(m, (size_t)st.st_size, MADV_SEQUENTIAL);
                q->map = (const char*)m;
                q->map_len = q->len = (size_t)st.st_size;
            }
        }
        if (!q->map && fd >= 0) {
            q->f = ::fdopen(fd, "rb");   // an empty file, a pipe, or a failed mapping
            if (!q->f) ::close(fd);
        } else if (fd >= 0) {
            ::close(fd);   // the mapping stays valid
        }
    }
    if (!q->map && !q->f && !q->gz && !q->bgzf) {
        delete q;
        return FAME_ERR_IO;
    }
    const int T = n_threads > 0 ? n_threads : (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    q->pool = new (std::nothrow) Pool(T);
    if (!q->pool) {
        fame_fastq_close(q);
        return FAME_ERR_NOMEM;
    }
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
        const uint32_t room = max_reads - n;
        // region: about the bytes of `room` records, whole lines
        size_t want = q->bytes_per_seq > 0 ? (size_t)(room * q->bytes_per_seq * 1.03) + (256u << 10) : BLOCK;
        if (!q->map && q->len - q->pos < want && !q->eof)
            if (!fill(q, std::max(want, BLOCK))) return FAME_ERR_IO;
        const char* base = data(q) + q->pos;
        const size_t avail = q->len - q->pos;
        if (avail == 0) break;
        size_t end = std::min(avail, want);
        if (end < avail) {
            const char* nl = (const char*)memrchr(base, '\n', end);
            if (nl) {
                end = (size_t)(nl - base) + 1;
            } else {   // one line longer than the region: take it whole
                nl = (const char*)std::memchr(base + end, '\n', avail - end);
                end = nl ? (size_t)(nl - base) + 1 : avail;
            }
        }
        if (end == avail && !at_end(q)) {   // buffered input: the last line may continue
            const char* nl = (const char*)memrchr(base, '\n', end);
            if (!nl) {
                if (!fill(q, BLOCK)) return FAME_ERR_IO;
                continue;
            }
            end = (size_t)(nl - base) + 1;
        }
        const uint32_t n0 = n;
        size_t consumed = 0;
        uint64_t lines = 0;
        const int rc = parse_region(q, base, end, room, seqs, seq_cap, offs, &n, &used, &consumed, &lines);
        if (rc) return rc;
        q->pos += consumed;
        q->line += lines;
        if (n > n0)
            q->bytes_per_seq = (double)consumed / (double)(n - n0);
        if (q->map) {   // release the pages behind the read position
            const size_t pg = (size_t)sysconf(_SC_PAGESIZE);
            const size_t upto = q->pos / pg * pg;
            if (upto > q->dropped + (64u << 20)) {
                ::madvise((void*)(q->map + q->dropped), upto - q->dropped, MADV_DONTNEED);
                q->dropped = upto;
            }
        }
        if (consumed < end) break;                      // stopped after max_reads records
        if (at_end(q) && q->pos >= q->len) break;
    }
    *n_out = n;
    return FAME_OK;
}

extern "C" int fame_fastq_close(fame_fastq* q)
{
    if (!q) return FAME_ERR_ARG;
    delete q->pool;
    if (q->map) ::munmap((void*)q->map, q->map_len);
    if (q->f) std::fclose(q->f);
    if (q->gz) gzclose(q->gz);
    if (q->bgzf) fame::bgzf_gpu_close(q->bgzf);
    if (q->cf) std::fclose(q->cf);
    delete q;
    return FAME_OK;
}

extern "C" int fame_fastq_gpu_inflate(const fame_fastq* q) { return q && q->bgzf ? 1 : 0; }
