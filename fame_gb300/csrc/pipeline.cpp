// FASTQ file to CpG tallies: queryRoutine (main.cpp:363-399) with parseChunk
// (ReadQueue.cpp:218-373) overlapped with the matching.  Chunks of CHUNKSIZE
// (or the caller's count of) records are parsed by the native reader straight into a free slot of a
// batched queue (its page-locked staging), so the host parses chunk i + 1
// while the GPU matches chunks i, i - 1, ...; the first chunk is matched
// alone with the strand vote (getStranded) unless both strands are queried,
// and decides matchR1Fwd for the rest as decideStrand (ReadQueue.cpp:376-400)
// does.  Tallies go to the context's array (or meth_dev); counters are summed
// over the chunks.  Results do not depend on the overlap: every read is
// matched alone and tallies and counters are sums.
#include <cstdint>
#include <deque>

#include "../../include/fame_gpu.h"

namespace {

constexpr uint32_t CHUNKSIZE = 300000;   // CONST.h:69

struct Closer {
    fame_fastq* f = nullptr;
    fame_queue* q = nullptr;
    ~Closer()
    {
        if (q) fame_queue_close(q);
        if (f) fame_fastq_close(f);
    }
};

// Parses the next chunk into a staged slot; n = 0 at the end of the input
// (the slot is then submitted empty, which records nothing).
int parse_into_slot(fame_queue* q, fame_fastq* f, uint32_t chunk, int* slot, uint32_t* n)
{
    char* seqs = nullptr;
    uint64_t* offs = nullptr;
    uint32_t max_reads = 0;
    uint64_t max_bytes = 0;
    int rc = fame_queue_stage(q, slot, &seqs, &offs, &max_reads, &max_bytes);
    if (rc) return rc;
    rc = fame_fastq_read(f, chunk < max_reads ? chunk : max_reads, seqs, max_bytes, offs, n);
    if (rc) fame_queue_submit_staged(q, *slot, 0, 0, nullptr);   // give the slot back
    return rc;
}

}  // namespace

extern "C" int fame_match_fastq(fame_gpu* g, const char* path, int is_gz, uint32_t flags, uint32_t chunk,
                                uint32_t slots, int n_threads, uint32_t* meth_dev, fame_counters* cnt,
                                uint64_t* n_reads)
{
    if (!g || !path || !cnt) return FAME_ERR_ARG;
    if (chunk == 0) chunk = CHUNKSIZE;
    if (slots < 2) slots = 2;
    if (slots > 8) slots = 8;
    *cnt = fame_counters{};
    if (n_reads) *n_reads = 0;
    Closer c;
    int rc = fame_fastq_open(path, is_gz, n_threads, &c.f);
    if (rc) return rc;
    rc = fame_queue_open(g, slots, chunk, (uint64_t)chunk * FAME_MAX_READ_LEN, &c.q);
    if (rc) return rc;
    const bool both = (flags & FAME_BOTH_STRANDS) != 0;
    bool match_r1_fwd = true;
    uint64_t total = 0;
    int slot = -1;
    uint32_t n = 0;
    if (!both) {
        // chunk 0 alone: its strand vote decides the orientation of the others
        if ((rc = parse_into_slot(c.q, c.f, chunk, &slot, &n))) return rc;
        if ((rc = fame_queue_submit_staged(c.q, slot, n, FAME_GET_STRANDED | FAME_MATCH_R1_FWD, meth_dev))) return rc;
        if ((rc = fame_queue_collect(c.q, slot, nullptr, nullptr, cnt))) return rc;
        total += n;
        match_r1_fwd = cnt->r1_fwd > cnt->r1_rev;
        if (n < chunk) {
            if (n_reads) *n_reads = total;
            return FAME_OK;
        }
    }
    const uint32_t later = (both ? FAME_BOTH_STRANDS : 0u) | (match_r1_fwd ? FAME_MATCH_R1_FWD : 0u);
    std::deque<int> inflight;
    for (;;) {
        if (inflight.size() == slots) {   // every slot busy: the oldest chunk finishes first
            if ((rc = fame_queue_collect(c.q, inflight.front(), nullptr, nullptr, cnt))) return rc;
            inflight.pop_front();
        }
        if ((rc = parse_into_slot(c.q, c.f, chunk, &slot, &n))) return rc;
        if ((rc = fame_queue_submit_staged(c.q, slot, n, later, meth_dev))) return rc;
        if (n == 0) {
            if ((rc = fame_queue_collect(c.q, slot, nullptr, nullptr, cnt))) return rc;
            break;
        }
        inflight.push_back(slot);
        total += n;
        if (n < chunk) break;
    }
    while (!inflight.empty()) {
        if ((rc = fame_queue_collect(c.q, inflight.front(), nullptr, nullptr, cnt))) return rc;
        inflight.pop_front();
    }
    if (n_reads) *n_reads = total;
    return FAME_OK;
}
