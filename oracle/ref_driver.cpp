// Test infrastructure only: a C API around the reference FAME sources, compiled
// from the reference's own files (staged under oracle/_ref/src by build_ref.sh).
//
// It exists to (1) generate golden vectors from the real reference for the
// parity tests, (2) validate the C restatement in fame_oracle.c and (3) time
// the reference's OpenMP matching path as the CPU baseline.  Nothing in the
// product links this file.
//
// The reference keeps its matching internals private and inline
// (ReadQueue.h:135-380); this translation unit is compiled with
// -Dprivate=public and includes ReadQueue.cpp so that getSeedRefs and the
// per-thread hopscotch maps can be inspected.

#include <unistd.h>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <fstream>
#include <string>
#include <vector>
#include <algorithm>

#include "ReadQueue.cpp"
#include "RefReader_istr.h"

namespace {

// The reference has no default constructor for RefGenome (RefGenome.h:45).
// RefGenome(std::string) runs load() (RefGenome.cpp:77-80); feed it a stub index
// with the right header constants and empty tables, then fill the members.
std::string write_stub_index()
{
    char tmpl[] = "/tmp/fame_ref_stubXXXXXX";
    int fd = mkstemp(tmpl);
    if (fd < 0) return std::string();
    close(fd);
    std::string path(tmpl);
    std::ofstream of(path, std::ofstream::binary | std::ofstream::trunc);
    uint64_t htabs = MyConst::HTABSIZE;
    uint32_t readl = MyConst::READLEN, winl = MyConst::WINLEN, kmerl = MyConst::KMERLEN;
    uint64_t kmerc = MyConst::KMERCUTOFF;
    uint32_t seedbits = MyConst::SEEDBITS;
    uint64_t zero = 0;
    of.write(reinterpret_cast<char*>(&htabs), 8);
    of.write(reinterpret_cast<char*>(&readl), 4);
    of.write(reinterpret_cast<char*>(&winl), 4);
    of.write(reinterpret_cast<char*>(&kmerl), 4);
    of.write(reinterpret_cast<char*>(&kmerc), 8);
    of.write(reinterpret_cast<char*>(&seedbits), 4);
    for (int i = 0; i < 10; ++i) of.write(reinterpret_cast<char*>(&zero), 8);
    of.close();
    std::ofstream os(path + "_strands", std::ofstream::binary | std::ofstream::trunc);
    os.write(reinterpret_cast<char*>(&zero), 8);
    os.close();
    return path;
}

RefGenome* empty_genome()
{
    std::string p = write_stub_index();
    if (p.empty()) return nullptr;
    RefGenome* r = new RefGenome(p);
    unlink(p.c_str());
    unlink((p + "_strands").c_str());
    return r;
}

// Mirror of RefGenome::save (RefGenome.cpp:144-153): the loaded index keeps
// only the upper 32 bits of each k-mer plus its T mask.
void small_from_full(RefGenome& r)
{
    r.kmerTableSmall.resize(r.kmerTable.size());
    for (size_t i = 0; i < r.kmerTable.size(); ++i)
        r.kmerTableSmall[i] = KMER_S::constructKmerS(KMER::getCore(r.kmerTable[i]), r.getTMask(r.kmerTable[i]));
    std::vector<KMER::kmer>().swap(r.kmerTable);
}

// ReadQueue opens errOut.txt in the working directory (ReadQueue.cpp:37);
// construct it from inside /tmp so no stray file lands in the caller's tree.
template <class F>
auto in_tmp(F f) -> decltype(f())
{
    char cwd[4096];
    char* ok = getcwd(cwd, sizeof(cwd));
    if (chdir("/tmp") != 0) {}
    auto r = f();
    if (ok && chdir(cwd) != 0) {}
    return r;
}

} // namespace

extern "C" {

int fame_ref_corenum() { return CORENUM; }
int fame_ref_readlen() { return (int)MyConst::READLEN; }

// Build the index the way main.cpp does (main.cpp:325-333): readReference + RefGenome ctor.
void* fame_ref_build(const char* fasta, int noloss)
{
    std::vector<struct CpG> cpgTab, cpgStartTab;
    std::vector<std::vector<char>> genSeq;
    std::unordered_map<uint8_t, std::string> chrMap;
    readReference(fasta, cpgTab, cpgStartTab, genSeq, chrMap, false);
    RefGenome* r = new RefGenome(std::move(cpgTab), std::move(cpgStartTab), genSeq, noloss != 0, chrMap);
    small_from_full(*r);
    return r;
}

// Build the index as main.cpp does and write it with the reference's own
// RefGenome::save (main.cpp:325-343, RefGenome.cpp:83-228).
int fame_ref_build_save(const char* fasta, int noloss, const char* path)
{
    std::vector<struct CpG> cpgTab, cpgStartTab;
    std::vector<std::vector<char>> genSeq;
    std::unordered_map<uint8_t, std::string> chrMap;
    readReference(fasta, cpgTab, cpgStartTab, genSeq, chrMap, false);
    RefGenome r(std::move(cpgTab), std::move(cpgStartTab), genSeq, noloss != 0, chrMap);
    r.save(path);
    return 0;
}

// Load an index written by RefGenome::save (--load_index path, RefGenome.cpp:230-387).
void* fame_ref_load(const char* path)
{
    return new RefGenome(std::string(path));
}

// Construct from raw arrays in the loaded-index layout (used to time the
// reference on an index produced elsewhere without an 8 GB file round trip).
void* fame_ref_from_arrays(uint32_t n_chrom, const char* const* chrom_seq, const uint64_t* chrom_len,
                           const char* const* chrom_name,
                           uint64_t n_cpg, const uint8_t* cpg_chrom, const uint32_t* cpg_pos,
                           uint64_t n_cpg_start, const uint8_t* cpgs_chrom, const uint32_t* cpgs_pos,
                           const uint64_t* tab_index /* HTABSIZE+1 */,
                           uint64_t n_kmer, const uint32_t* kmer_meta, const uint32_t* kmer_tmask,
                           const uint8_t* strand,
                           uint64_t n_win, const uint32_t* win_start, const uint8_t* win_chrom,
                           const uint32_t* win_sind, const uint32_t* win_eind,
                           uint64_t n_filtered, const uint64_t* filtered)
{
    RefGenome* r = empty_genome();
    if (!r) return nullptr;
    r->fullSeq.resize(n_chrom);
    for (uint32_t c = 0; c < n_chrom; ++c) {
        r->fullSeq[c].assign(chrom_seq[c], chrom_seq[c] + chrom_len[c]);
        r->chrMap[(uint8_t)c] = chrom_name ? std::string(chrom_name[c]) : std::to_string(c);
    }
    r->cpgTable.resize(n_cpg);
    for (uint64_t i = 0; i < n_cpg; ++i) r->cpgTable[i] = {cpg_chrom[i], cpg_pos[i]};
    r->cpgStartTable.resize(n_cpg_start);
    for (uint64_t i = 0; i < n_cpg_start; ++i) r->cpgStartTable[i] = {cpgs_chrom[i], cpgs_pos[i]};
    r->tabIndex.assign(tab_index, tab_index + MyConst::HTABSIZE + 1);
    r->kmerTableSmall.resize(n_kmer);
    r->strandTable.resize(n_kmer);
    for (uint64_t i = 0; i < n_kmer; ++i) {
        r->kmerTableSmall[i] = KMER_S::constructKmerS(kmer_meta[i], kmer_tmask ? kmer_tmask[i] : 0);
        r->strandTable[i] = strand[i] != 0;
    }
    r->metaWindows.resize(n_win);
    for (uint64_t i = 0; i < n_win; ++i) r->metaWindows[i] = {win_start[i], win_chrom[i], win_sind[i], win_eind[i]};
    for (uint64_t i = 0; i < n_filtered; ++i) r->filteredKmers.emplace(filtered[i]);
    return r;
}

void fame_ref_free(void* ref) { delete static_cast<RefGenome*>(ref); }

// Sizes of the index tables (for sizing the dump buffers).
void fame_ref_sizes(void* ref, uint64_t* out /* 7 */)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    uint64_t nonempty = 0;
    for (uint64_t i = 0; i < MyConst::HTABSIZE; ++i) nonempty += (r.tabIndex[i + 1] != r.tabIndex[i]);
    out[0] = r.cpgTable.size();
    out[1] = r.cpgStartTable.size();
    out[2] = r.fullSeq.size();
    out[3] = nonempty;
    out[4] = r.kmerTableSmall.size();
    out[5] = r.metaWindows.size();
    out[6] = r.filteredKmers.size();
}

// Dump the loaded-index tables; buffers sized from fame_ref_sizes.
void fame_ref_dump(void* ref, uint8_t* cpg_chrom, uint32_t* cpg_pos, uint8_t* cpgs_chrom, uint32_t* cpgs_pos,
                   uint32_t* bucket_key, uint64_t* bucket_start, uint32_t* bucket_len,
                   uint32_t* kmer_meta, uint32_t* kmer_tmask, uint8_t* strand,
                   uint32_t* win_start, uint8_t* win_chrom, uint32_t* win_sind, uint32_t* win_eind,
                   uint64_t* filtered)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    for (size_t i = 0; i < r.cpgTable.size(); ++i) { cpg_chrom[i] = r.cpgTable[i].chrom; cpg_pos[i] = r.cpgTable[i].pos; }
    for (size_t i = 0; i < r.cpgStartTable.size(); ++i) { cpgs_chrom[i] = r.cpgStartTable[i].chrom; cpgs_pos[i] = r.cpgStartTable[i].pos; }
    uint64_t b = 0;
    for (uint64_t i = 0; i < MyConst::HTABSIZE; ++i) {
        if (r.tabIndex[i + 1] != r.tabIndex[i]) {
            bucket_key[b] = (uint32_t)i;
            bucket_start[b] = r.tabIndex[i];
            bucket_len[b] = (uint32_t)(r.tabIndex[i + 1] - r.tabIndex[i]);
            ++b;
        }
    }
    for (size_t i = 0; i < r.kmerTableSmall.size(); ++i) {
        kmer_meta[i] = r.kmerTableSmall[i].meta;
        kmer_tmask[i] = r.kmerTableSmall[i].tmask;
        strand[i] = r.strandTable[i] ? 1 : 0;
    }
    for (size_t i = 0; i < r.metaWindows.size(); ++i) {
        win_start[i] = r.metaWindows[i].startPos; win_chrom[i] = r.metaWindows[i].chrom;
        win_sind[i] = r.metaWindows[i].startInd; win_eind[i] = r.metaWindows[i].endInd;
    }
    std::vector<uint64_t> f(r.filteredKmers.begin(), r.filteredKmers.end());
    std::sort(f.begin(), f.end());
    std::copy(f.begin(), f.end(), filtered);
}

// Single-end run with the loop structure of queryRoutine (main.cpp:363-399):
// chunk 0 is matched with getStranded unless both_strands, then decideStrand;
// the remaining chunks only in the decided orientation.  parseChunk's
// `readBuffer[i] = Read(seq, id)` (ReadQueue.cpp:233) is reproduced directly.
//
// counters: [succ, nonunique, unsucc, r1Fwd, r1Rev, matchR1Fwd]
int fame_ref_match_se(void* ref, const char* seqs, const uint64_t* offs, uint32_t n, uint32_t chunk,
                      int both_strands, uint64_t* mats, uint8_t* invalid, uint16_t* meth,
                      uint64_t* counters, double* seconds)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    ReadQueue* rq = in_tmp([&] { return new ReadQueue("/dev/null", r, false, both_strands != 0); });
    if (chunk == 0 || chunk > MyConst::CHUNKSIZE) chunk = MyConst::CHUNKSIZE;
    uint64_t succ = 0, nonu = 0, unsucc = 0;
    double secs = 0.0;
    std::string id("r");
    for (uint32_t c0 = 0, ci = 0; c0 < n || (c0 == 0 && n == 0); c0 += chunk, ++ci) {
        const uint32_t cn = std::min<uint32_t>(chunk, n - c0);
        for (uint32_t j = 0; j < cn; ++j) {
            std::string s(seqs + offs[c0 + j], seqs + offs[c0 + j + 1]);
            rq->readBuffer[j] = Read(s, id);
        }
        const bool stranded = (ci == 0) && !both_strands;
        auto t0 = std::chrono::steady_clock::now();
        rq->matchReads(cn, succ, nonu, unsucc, stranded);
        auto t1 = std::chrono::steady_clock::now();
        secs += std::chrono::duration<double>(t1 - t0).count();
        if (stranded) rq->decideStrand();
        for (uint32_t j = 0; j < cn; ++j) {
            invalid[c0 + j] = rq->readBuffer[j].isInvalid ? 1 : 0;
            mats[c0 + j] = rq->readBuffer[j].isInvalid ? 0 : rq->readBuffer[j].mat;
        }
        if (n == 0) break;
    }
    for (size_t i = 0; i < r.cpgTable.size(); ++i) {
        meth[4 * i + 0] = rq->methLevels[i].methFwd;
        meth[4 * i + 1] = rq->methLevels[i].unmethFwd;
        meth[4 * i + 2] = rq->methLevels[i].methRev;
        meth[4 * i + 3] = rq->methLevels[i].unmethRev;
    }
    counters[0] = succ; counters[1] = nonu; counters[2] = unsucc;
    counters[3] = rq->r1FwdMatches; counters[4] = rq->r1RevMatches; counters[5] = rq->matchR1Fwd ? 1 : 0;
    if (seconds) *seconds = secs;
    delete rq;
    return 0;
}

// getSeedRefs for one sequence (ReadQueue.cpp:2325-2461) and the resulting
// hopscotch map contents in iteration order.  out_keys/out_counts hold the
// forward map first (n_out[0] entries) then the reverse map (n_out[1]);
// n_out[2], n_out[3] are the final bucket counts of the two maps.
int fame_ref_seed_order(void* ref, const char* seq, uint32_t len, uint32_t cap,
                        uint32_t* out_keys, uint32_t* out_counts, uint64_t* n_out)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    ReadQueue* rq = in_tmp([&] { return new ReadQueue("/dev/null", r, false, true); });
    std::string s(seq, seq + len);
    rq->getSeedRefs(s, s.size(), MyConst::QTHRESH);
    uint32_t k = 0;
    uint64_t nf = 0, nr = 0;
    for (const auto& m : rq->fwdMetaIDs[0]) { if (k < cap) { out_keys[k] = m.first; out_counts[k] = m.second; } ++k; ++nf; }
    for (const auto& m : rq->revMetaIDs[0]) { if (k < cap) { out_keys[k] = m.first; out_counts[k] = m.second; } ++k; ++nr; }
    n_out[0] = nf; n_out[1] = nr;
    n_out[2] = rq->fwdMetaIDs[0].bucket_count();
    n_out[3] = rq->revMetaIDs[0].bucket_count();
    delete rq;
    return k > cap ? -1 : 0;
}

// The reference's own LevenshtDP (LevenshtDP.h:191-544) on one read/reference
// pair with FAME's comparators (ReadQueue.h:295-338) or a plain equality
// comparator (LevenshtDP_unittest.cpp), for pinning the DP restatement.
// comp: 0 = equality, 1 = CompiFwd, 2 = CompiRev, 3 = plain complement (unit test simpleSeqRev)
// rev: 0 = runDPFill/backtrackDP, 1 = runDPFillRev/backtrackDPRev
} // extern "C"
struct EqComp { uint16_t operator()(const char a, const char b) { return a == b ? 0 : 1; } };
struct ComplComp {
    uint16_t operator()(const char c1, const char c2) {
        switch (c1) {
            case 'A': return c2 == 'T' ? 0 : 1;
            case 'C': return c2 == 'G' ? 0 : 1;
            case 'G': return c2 == 'C' ? 0 : 1;
            case 'T': return c2 == 'A' ? 0 : 1;
        }
        return 1;
    }
};
template <size_t B, class C>
static int run_lev(const std::string& row, const char* col, int rev, C comp, uint8_t* trace, uint32_t cap, uint32_t* dist)
{
    LevenshtDP<uint16_t, B> lev(row, col);
    std::vector<ERROR_T> al;
    if (rev) { lev.template runDPFillRev<C>(comp); *dist = lev.getEditDist(); lev.template backtrackDPRev<C>(comp, al); }
    else { lev.template runDPFill<C>(comp); *dist = lev.getEditDist(); lev.template backtrackDP<C>(comp, al); }
    for (size_t i = 0; i < al.size() && i < cap; ++i) trace[i] = (uint8_t)al[i];
    return (int)al.size();
}
template <size_t B>
static int lev_dispatch(const std::string& row, const char* col, int rev, int comp, uint8_t* trace, uint32_t cap, uint32_t* dist)
{
    ReadQueue::CompiFwd cf; ReadQueue::CompiRev cr;
    switch (comp) {
        case 0: return run_lev<B>(row, col, rev, EqComp(), trace, cap, dist);
        case 1: return run_lev<B>(row, col, rev, cf, trace, cap, dist);
        case 2: return run_lev<B>(row, col, rev, cr, trace, cap, dist);
        default: return run_lev<B>(row, col, rev, ComplComp(), trace, cap, dist);
    }
}
extern "C" {
int fame_ref_lev(int band, const char* row, uint32_t row_len, const char* col_end, int rev, int comp,
                 uint8_t* trace, uint32_t cap, uint32_t* dist)
{
    std::string r(row, row + row_len);
    switch (band) {
        case 0: return lev_dispatch<0>(r, col_end, rev, comp, trace, cap, dist);
        case 1: return lev_dispatch<1>(r, col_end, rev, comp, trace, cap, dist);
        case 2: return lev_dispatch<2>(r, col_end, rev, comp, trace, cap, dist);
        case 8: return lev_dispatch<8>(r, col_end, rev, comp, trace, cap, dist);
    }
    return -1;
}

// The reference ShiftAnd (ShiftAnd.h) on one text window: fwd = querySeq over
// [text, text+len), rev = queryRevSeq from text+len-1 down to (excl.) text-1.
int fame_ref_shiftand(const char* pat, uint32_t pat_len, const char* text, uint32_t text_len, int rev,
                      uint64_t* offs, uint8_t* errs, uint32_t cap)
{
    std::array<uint8_t, 16> lmap;
    lmap['A' % 16] = 0; lmap['C' % 16] = 1; lmap['G' % 16] = 2; lmap['T' % 16] = 3;
    std::string p(pat, pat + pat_len);
    ShiftAnd<MyConst::MISCOUNT + MyConst::ADDMIS> sa(p, lmap);
    std::vector<char> t(text_len + 1, 'N');
    std::copy(text, text + text_len, t.begin() + 1);
    std::vector<uint64_t> m;
    std::vector<uint8_t> e;
    if (rev) sa.queryRevSeq(t.begin() + text_len, t.begin(), m, e);
    else sa.querySeq(t.begin() + 1, t.begin() + 1 + text_len, m, e);
    for (size_t i = 0; i < m.size() && i < cap; ++i) { offs[i] = m[i]; errs[i] = e[i]; }
    return (int)m.size();
}

} // extern "C"

extern "C" {
// Insert keys with operator[] (as getSeedRefs does, ReadQueue.cpp:2392-2400)
// into a tsl::hopscotch_map built with `bucket_count` (ReadQueue.cpp:2356) and
// return the iteration order; pins the insertion model of the oracle.
int fame_ref_hopscotch(const uint32_t* keys, uint32_t n, uint32_t bucket_count, uint32_t* order, uint64_t* final_buckets)
{
    tsl::hopscotch_map<uint32_t, uint16_t, ReadQueue::MetaHash> m(bucket_count);
    for (uint32_t i = 0; i < n; ++i) ++m[keys[i]];
    uint32_t k = 0;
    for (const auto& e : m) order[k++] = e.first;
    *final_buckets = m.bucket_count();
    return (int)k;
}
}

extern "C" {
// Steady-state timing of ReadQueue::matchReads (ReadQueue.cpp:404-933): the
// orientation is already decided (matchR1Fwd given, getStranded false), as for
// every chunk after the first in queryRoutine (main.cpp:383-388).  Only the
// matchReads calls are timed.  counters: [succ, nonunique, unsucc].  When
// given (non-null), mats / invalid receive each read's MATCH::match (0 when
// invalid) and isInvalid, and meth the methLevels of the run (4 per CpG),
// all read after the timed calls.
int fame_ref_time_se(void* ref, const char* seqs, const uint64_t* offs, uint32_t n, int both_strands,
                     int match_r1_fwd, uint64_t* counters, double* seconds, uint64_t* mats, uint8_t* invalid,
                     uint16_t* meth)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    ReadQueue* rq = in_tmp([&] { return new ReadQueue("/dev/null", r, false, both_strands != 0); });
    rq->matchR1Fwd = match_r1_fwd != 0;
    uint64_t succ = 0, nonu = 0, unsucc = 0;
    double secs = 0.0;
    std::string id("r");
    const uint32_t chunk = MyConst::CHUNKSIZE;
    for (uint32_t c0 = 0; c0 < n; c0 += chunk) {
        const uint32_t cn = std::min<uint32_t>(chunk, n - c0);
        for (uint32_t j = 0; j < cn; ++j) {
            std::string s(seqs + offs[c0 + j], seqs + offs[c0 + j + 1]);
            rq->readBuffer[j] = Read(s, id);
        }
        auto t0 = std::chrono::steady_clock::now();
        rq->matchReads(cn, succ, nonu, unsucc, false);
        auto t1 = std::chrono::steady_clock::now();
        secs += std::chrono::duration<double>(t1 - t0).count();
        if (mats && invalid)
            for (uint32_t j = 0; j < cn; ++j) {
                invalid[c0 + j] = rq->readBuffer[j].isInvalid ? 1 : 0;
                mats[c0 + j] = rq->readBuffer[j].isInvalid ? 0 : rq->readBuffer[j].mat;
            }
    }
    if (meth)
        for (size_t i = 0; i < r.cpgTable.size(); ++i) {
            meth[4 * i + 0] = rq->methLevels[i].methFwd;
            meth[4 * i + 1] = rq->methLevels[i].unmethFwd;
            meth[4 * i + 2] = rq->methLevels[i].methRev;
            meth[4 * i + 3] = rq->methLevels[i].unmethRev;
        }
    counters[0] = succ; counters[1] = nonu; counters[2] = unsucc;
    *seconds = secs;
    delete rq;
    return 0;
}
}

extern "C" {
int fame_ref_maxpdist() { return (int)MyConst::MAXPDIST; }

// Paired-end run with the loop structure of queryRoutinePaired (main.cpp:400-441):
// chunk 0 with getStranded unless both_strands, decideStrand, later chunks in the
// decided orientation.  counters: [succ, nonunique, unsucc, succPaired, tooShort,
// r1Fwd, r1Rev, matchR1Fwd]
int fame_ref_match_pe(void* ref, const char* s1, const uint64_t* o1, const char* s2, const uint64_t* o2, uint32_t n,
                      uint32_t chunk, int both_strands, uint64_t* mats1, uint64_t* mats2, uint8_t* inv1,
                      uint8_t* inv2, uint16_t* meth, uint64_t* counters, double* seconds)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    ReadQueue* rq = in_tmp([&] { return new ReadQueue("/dev/null", "/dev/null", r, false, both_strands != 0); });
    if (chunk == 0 || chunk > MyConst::CHUNKSIZE) chunk = MyConst::CHUNKSIZE;
    uint64_t succ = 0, nonu = 0, unsucc = 0, paired = 0, tooShort = 0;
    double secs = 0.0;
    std::string id("r");
    for (uint32_t c0 = 0, ci = 0; c0 < n; c0 += chunk, ++ci) {
        const uint32_t cn = std::min<uint32_t>(chunk, n - c0);
        for (uint32_t j = 0; j < cn; ++j) {
            std::string a(s1 + o1[c0 + j], s1 + o1[c0 + j + 1]);
            std::string b(s2 + o2[c0 + j], s2 + o2[c0 + j + 1]);
            rq->readBuffer[j] = Read(a, id);
            rq->readBuffer2[j] = Read(b, id);
        }
        const bool stranded = (ci == 0) && !both_strands;
        auto t0 = std::chrono::steady_clock::now();
        rq->matchPairedReads(cn, succ, nonu, unsucc, paired, tooShort, stranded);
        auto t1 = std::chrono::steady_clock::now();
        secs += std::chrono::duration<double>(t1 - t0).count();
        if (stranded) rq->decideStrand();
        for (uint32_t j = 0; j < cn; ++j) {
            inv1[c0 + j] = rq->readBuffer[j].isInvalid ? 1 : 0;
            inv2[c0 + j] = rq->readBuffer2[j].isInvalid ? 1 : 0;
            mats1[c0 + j] = rq->readBuffer[j].isInvalid ? 0 : rq->readBuffer[j].mat;
            mats2[c0 + j] = rq->readBuffer2[j].isInvalid ? 0 : rq->readBuffer2[j].mat;
        }
    }
    for (size_t i = 0; i < r.cpgTable.size(); ++i) {
        meth[4 * i + 0] = rq->methLevels[i].methFwd;
        meth[4 * i + 1] = rq->methLevels[i].unmethFwd;
        meth[4 * i + 2] = rq->methLevels[i].methRev;
        meth[4 * i + 3] = rq->methLevels[i].unmethRev;
    }
    counters[0] = succ; counters[1] = nonu; counters[2] = unsucc; counters[3] = paired; counters[4] = tooShort;
    counters[5] = rq->r1FwdMatches; counters[6] = rq->r1RevMatches; counters[7] = rq->matchR1Fwd ? 1 : 0;
    if (seconds) *seconds = secs;
    delete rq;
    return 0;
}

// Seconds spent in matchPairedReads for already-stranded chunks (the steady
// state of queryRoutinePaired after decideStrand); counters: [succ, nonunique,
// unsucc, succPaired, tooShort].  When given (non-null), mats (2n: mate 1
// then mate 2 of each pair, 0 when invalid), invalid (2n, same order) and meth
// (4 per CpG) receive the run's results, read after the timed calls.
int fame_ref_time_pe(void* ref, const char* s1, const uint64_t* o1, const char* s2, const uint64_t* o2, uint32_t n,
                     int both_strands, int match_r1_fwd, uint64_t* counters, double* seconds, uint64_t* mats,
                     uint8_t* invalid, uint16_t* meth)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    ReadQueue* rq = in_tmp([&] { return new ReadQueue("/dev/null", "/dev/null", r, false, both_strands != 0); });
    rq->matchR1Fwd = match_r1_fwd != 0;
    uint64_t succ = 0, nonu = 0, unsucc = 0, paired = 0, tooShort = 0;
    double secs = 0.0;
    std::string id("r");
    const uint32_t chunk = MyConst::CHUNKSIZE;
    for (uint32_t c0 = 0; c0 < n; c0 += chunk) {
        const uint32_t cn = std::min<uint32_t>(chunk, n - c0);
        for (uint32_t j = 0; j < cn; ++j) {
            std::string a(s1 + o1[c0 + j], s1 + o1[c0 + j + 1]);
            std::string b(s2 + o2[c0 + j], s2 + o2[c0 + j + 1]);
            rq->readBuffer[j] = Read(a, id);
            rq->readBuffer2[j] = Read(b, id);
        }
        auto t0 = std::chrono::steady_clock::now();
        rq->matchPairedReads(cn, succ, nonu, unsucc, paired, tooShort, false);
        auto t1 = std::chrono::steady_clock::now();
        secs += std::chrono::duration<double>(t1 - t0).count();
        if (mats && invalid)
            for (uint32_t j = 0; j < cn; ++j) {
                const Read& a = rq->readBuffer[j];
                const Read& b = rq->readBuffer2[j];
                invalid[c0 + j] = a.isInvalid ? 1 : 0;
                invalid[n + c0 + j] = b.isInvalid ? 1 : 0;
                mats[c0 + j] = a.isInvalid ? 0 : a.mat;
                mats[n + c0 + j] = b.isInvalid ? 0 : b.mat;
            }
    }
    if (meth)
        for (size_t i = 0; i < r.cpgTable.size(); ++i) {
            meth[4 * i + 0] = rq->methLevels[i].methFwd;
            meth[4 * i + 1] = rq->methLevels[i].unmethFwd;
            meth[4 * i + 2] = rq->methLevels[i].methRev;
            meth[4 * i + 3] = rq->methLevels[i].unmethRev;
        }
    counters[0] = succ; counters[1] = nonu; counters[2] = unsucc; counters[3] = paired; counters[4] = tooShort;
    *seconds = secs;
    delete rq;
    return 0;
}

// std::sort with the paired path's comparator (cmpMetaFirst, ReadQueue.h:340-346):
// input in the given order, output the keys in sorted order (pins the tie order).
int fame_ref_sort_desc(const uint32_t* keys, const uint8_t* counts, uint32_t n, uint32_t* out)
{
    std::vector<std::pair<uint32_t, std::tuple<uint8_t, uint8_t, bool, bool>>> v;
    for (uint32_t i = 0; i < n; ++i) v.push_back({keys[i], std::make_tuple(counts[i], (uint8_t)0, false, false)});
    ReadQueue::CompiMetaFirst c;
    std::sort(v.begin(), v.end(), c);
    for (uint32_t i = 0; i < n; ++i) out[i] = v[i].first;
    return 0;
}
}

extern "C" {
// printMethylationLevels (ReadQueue.cpp:1860-1893) of the given tallies (4
// uint16 per CpG in cpgTable order): writes <basename>_cpg.tsv.
int fame_ref_print_cpg(void* ref, const uint16_t* meth, const char* basename)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    ReadQueue* rq = in_tmp([&] { return new ReadQueue("/dev/null", r, false, false); });
    for (size_t i = 0; i < r.cpgTable.size(); ++i) {
        rq->methLevels[i].methFwd = meth[4 * i + 0];
        rq->methLevels[i].unmethFwd = meth[4 * i + 1];
        rq->methLevels[i].methRev = meth[4 * i + 2];
        rq->methLevels[i].unmethRev = meth[4 * i + 3];
    }
    std::string fn(basename);
    rq->printMethylationLevels(fn);
    delete rq;
    return 0;
}

// The single-cell matrix: the single-cell ReadQueue's header
// (ReadQueue.cpp:182-215) and printSCMethylationLevels (1894-1921) for each
// of n cells (ids[c], tallies meth + 4 * n_cpg * c), written to path.
int fame_ref_print_sc(void* ref, const char* path, uint32_t n, const char* const* ids, const uint16_t* meth)
{
    RefGenome& r = *static_cast<RefGenome*>(ref);
    ReadQueue* rq = in_tmp([&] { return new ReadQueue(path, r, false, false, false); });
    const size_t nc = r.cpgTable.size();
    for (uint32_t c = 0; c < n; ++c) {
        for (size_t i = 0; i < nc; ++i) {
            rq->methLevels[i].methFwd = meth[4 * (nc * c + i) + 0];
            rq->methLevels[i].unmethFwd = meth[4 * (nc * c + i) + 1];
            rq->methLevels[i].methRev = meth[4 * (nc * c + i) + 2];
            rq->methLevels[i].unmethRev = meth[4 * (nc * c + i) + 3];
        }
        rq->printSCMethylationLevels(std::string(ids[c]));
    }
    delete rq;
    return 0;
}
}
