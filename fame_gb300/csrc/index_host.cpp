// Host side of the index boundary: the --load_index file reader and a
// multi-threaded index builder producing the same tables as the reference's
// RefGenome constructor (RefReader_istr.h:48-113, RefGenome.cpp:26-74,
// 532-759, 1787-1989, 2191-2352) and save() (RefGenome.cpp:83-228).
//
// The builder keeps the reference's table contents and order exactly: within
// a hash bucket the entries appear in reverse insertion order (the reference
// fills by decrementing tabIndex, RefGenome.cpp:711-755), insertion order
// being window, then N-free interval, then reverse strand before forward,
// then k-mer position.  It parallelises the two hashing passes over windows
// with atomic bucket counters and restores that order with a per-bucket sort.
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/fame_gpu.h"
#include "fame_const.h"
#include "index_host.h"

using namespace fame;

namespace {

inline uint64_t rotl64(uint64_t v, unsigned s) { s &= 63u; return s ? (v << s) | (v >> (64 - s)) : v; }

// msTab (spaced_nthash/nthash.hpp:88-121)
inline uint64_t nt_val(uint8_t c)
{
    switch (c) {
        case 'A': case 'a': case 4: return NT_SEED_A;
        case 'C': case 'c': case 'T': case 't': case 1: case 7: return NT_SEED_T;
        case 'G': case 'g': case 3: return NT_SEED_G;
        default: return 0;
    }
}

// NTPS64 (nthash.hpp:480-498): full hash rolled, the four unseeded positions
// (SEEDBITS zeros at 2, 7, 14, 30) removed.
struct SpacedRoller {
    uint64_t h = 0;
    void init(const uint8_t* s) { h = 0; for (unsigned i = 0; i < KMERLEN; ++i) h ^= rotl64(nt_val(s[i]), 31 - i); }
    void roll(uint8_t out, uint8_t in) { h = rotl64(h, 1) ^ rotl64(nt_val(out), KMERLEN) ^ nt_val(in); }
    uint64_t spaced(const uint8_t* s) const
    {
        return h ^ rotl64(nt_val(s[2]), 29) ^ rotl64(nt_val(s[7]), 24) ^ rotl64(nt_val(s[14]), 17) ^ rotl64(nt_val(s[30]), 1);
    }
};

// fn(begin, end, part) over `threads` contiguous parts.  An exception thrown by
// a part is caught in its thread and rethrown here after every thread joined
// (so it reaches the entry point's handler instead of ending the process);
// parts whose thread cannot be started run on the calling thread.
template <class F>
void parallel_for(uint64_t n, int threads, F fn)
{
    if (threads <= 1 || n < 2) { fn(0, n, 0); return; }
    std::vector<std::thread> th;
    std::exception_ptr err;
    std::mutex err_mu;
    auto guarded = [&](uint64_t b, uint64_t e, int t) {
        try {
            fn(b, e, t);
        } catch (...) {
            std::lock_guard<std::mutex> lk(err_mu);
            if (!err) err = std::current_exception();
        }
    };
    const uint64_t step = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const uint64_t b = std::min<uint64_t>(n, t * step), e = std::min<uint64_t>(n, b + step);
        if (b >= e) break;
        try {
            th.emplace_back([=, &guarded] { guarded(b, e, t); });
        } catch (const std::system_error&) {
            guarded(b, e, t);
        }
    }
    for (auto& x : th) x.join();
    if (err) std::rethrow_exception(err);
}

// K-mers of one window in the reference's insertion order (RefGenome.cpp:621-759):
// emit(key, offset, strand).  red/redr are scratch of WINLEN bytes.
template <class Emit>
void window_kmers(const fame_host_index& ix, uint64_t w, uint8_t* red, uint8_t* redr, uint32_t* iv, Emit emit)
{
    memset(red, 0, WINLEN);
    memset(redr, 0, WINLEN);
    const fame_window& win = ix.win[w];
    const std::string& g = ix.seq[win.chrom];
    const uint64_t sp = win.start_pos;
    const uint64_t stop = std::min<uint64_t>(sp + WINLEN, g.size());
    bool lastN = true;
    uint32_t nStart = 0, niv = 0, j = 0;
    for (uint64_t i = sp; i < stop; ++i, ++j) {
        const uint32_t rp = WINLEN - 1 - j;
        switch (g[i]) {
            case 'N':
                if (!lastN) { iv[2 * niv] = nStart; iv[2 * niv + 1] = j - 1; ++niv; }
                lastN = true;
                red[j] = 'N';
                red[rp] = 'N';  // the reference writes the forward buffer here (RefGenome.cpp:646)
                break;
            case 'C': if (lastN) { nStart = j; lastN = false; } red[j] = 'T'; redr[rp] = 'G'; break;
            case 'G': if (lastN) { nStart = j; lastN = false; } red[j] = 'G'; redr[rp] = 'T'; break;
            case 'T': if (lastN) { nStart = j; lastN = false; } red[j] = 'T'; redr[rp] = 'A'; break;
            case 'A': if (lastN) { nStart = j; lastN = false; } red[j] = 'A'; redr[rp] = 'T'; break;
            default: break;
        }
    }
    if (!lastN) { iv[2 * niv] = nStart; iv[2 * niv + 1] = j - 1; ++niv; }
    SpacedRoller r;
    for (uint32_t q = 0; q < niv; ++q) {
        const uint32_t first = iv[2 * q], second = iv[2 * q + 1];
        const uint32_t dist = second - first + 1;
        if (dist < ix.readlen) continue;
        for (int strand = 0; strand < 2; ++strand) {  // reverse strand first
            const uint8_t* s = strand ? red + first : redr + (WINLEN - 1 - second);
            uint32_t kp = strand ? first : WINLEN - first - KMERLEN;
            r.init(s);
            emit((uint32_t)(r.spaced(s) & HTAB_MASK), kp, strand);
            for (uint32_t i = 0; i < dist - KMERLEN; ++i) {
                kp = strand ? kp + 1 : kp - 1;
                r.roll(s[i], s[i + KMERLEN]);
                if (i % SKIPMOD) continue;
                emit((uint32_t)(r.spaced(s + i + 1) & HTAB_MASK), kp, strand);
            }
        }
    }
}

inline uint8_t base_at(const fame_host_index& ix, uint32_t c, uint64_t p)
{
    return p < ix.seq[c].size() ? (uint8_t)ix.seq[c][p] : 'N';  // past the chromosome end: no base
}

// Fields of the builder's 64-bit bucket entries (window 63-32, insertion
// index 31-16, offset in the window 15-1, strand 0).
inline uint32_t ent_win(uint64_t e) { return (uint32_t)(e >> 32); }
inline uint32_t ent_off(uint64_t e) { return (uint32_t)(e >> 1) & 0x7fffu; }
inline int ent_fwd(uint64_t e) { return (int)(e & 1u); }

// reproduceKmerSeq (RefGenome.cpp:2028-2132)
uint64_t kmer_seq(const fame_host_index& ix, uint32_t w, uint32_t off, int fwd)
{
    const uint32_t c = ix.win[w].chrom;
    const uint64_t s0 = (uint64_t)ix.win[w].start_pos + off;
    uint64_t k = 0;
    for (unsigned i = 0; i < KMERLEN; ++i) {
        k <<= 2;  // the reverse loop of the reference walks i = 32..1 with SEED[32 - i], i.e. the same seed index
        if (!((SEEDBITS >> (31 - i)) & 1u)) continue;
        if (fwd) {
            const uint8_t ch = base_at(ix, c, s0 + i);
            if (ch == 'C' || ch == 'T') k += 3; else if (ch == 'G') k += 2;
        } else {
            const uint8_t ch = base_at(ix, c, s0 + KMERLEN - 1 - i);
            if (ch == 'G' || ch == 'A') k += 3; else if (ch == 'C') k += 2;
        }
    }
    return k;
}

// Per chromosome, one bit per base: 'T' most significant bit first in each
// 64-bit word, 'A' least significant bit first; positions past the end
// (and N) are 0, as base_at reads them.  The padding covers windows that
// reach WINLEN past a chromosome's end.
struct BaseBits {
    std::vector<std::vector<uint64_t>> t_msb, a_lsb;

    BaseBits(const fame_host_index& ix, int T) : t_msb(ix.seq.size()), a_lsb(ix.seq.size())
    {
        for (size_t c = 0; c < ix.seq.size(); ++c) {
            const uint64_t words = (ix.seq[c].size() + 2 * WINLEN) / 64 + 2;
            t_msb[c].assign(words, 0);
            a_lsb[c].assign(words, 0);
            const std::string& g = ix.seq[c];
            const uint64_t full = g.size() / 64 + 1;
            parallel_for(full, T, [&](uint64_t b, uint64_t e, int) {
                for (uint64_t wd = b; wd < e; ++wd) {
                    uint64_t t = 0, a = 0;
                    const uint64_t p0 = wd * 64, p1 = std::min<uint64_t>(p0 + 64, g.size());
                    for (uint64_t p = p0; p < p1; ++p) {
                        if (g[p] == 'T') t |= 1ull << (63 - (p - p0));
                        else if (g[p] == 'A') a |= 1ull << (p - p0);
                    }
                    t_msb[c][wd] = t;
                    a_lsb[c][wd] = a;
                }
            });
        }
    }
    // bit 31 - i: 'T' at s + i, i < 32
    uint32_t t_fwd(uint32_t c, uint64_t s) const
    {
        const std::vector<uint64_t>& b = t_msb[c];
        const uint64_t w = s >> 6, r = s & 63;
        const uint64_t x = r ? (b[w] << r) | (b[w + 1] >> (64 - r)) : b[w];
        return (uint32_t)(x >> 32);
    }
    // bit j: 'A' at s + j, j < 32
    uint32_t a_lo(uint32_t c, uint64_t s) const
    {
        const std::vector<uint64_t>& b = a_lsb[c];
        const uint64_t w = s >> 6, r = s & 63;
        const uint64_t x = r ? (b[w] >> r) | (b[w + 1] << (64 - r)) : b[w];
        return (uint32_t)x;
    }
};

// reproduceTMask (RefGenome.cpp:2135-2189): forward, bit 31 - i is 'T' at
// s0 + i; reverse, bit 31 - i is 'A' at s0 + 31 - i, i.e. bit j is 'A' at s0 + j.
uint32_t tmask_repro(const fame_host_index& ix, const BaseBits& bb, uint32_t w, uint32_t off, int fwd)
{
    const uint32_t c = ix.win[w].chrom;
    const uint64_t s0 = (uint64_t)ix.win[w].start_pos + off;
    return fwd ? bb.t_fwd(c, s0) : bb.a_lo(c, s0);
}

}  // namespace

// ---------------------------------------------------------------------------
// builder
// ---------------------------------------------------------------------------
// readReference and generateWindows: normalised sequences, CpG tables and
// windows (shared by the host and the device builder).
void fame::index_build_front(fame_host_index* ix, uint32_t readlen, uint32_t n_chrom, const char* const* seq,
                             const uint64_t* len, const char* const* names, int T)
{
    ix->readlen = readlen;
    ix->seq.resize(n_chrom);
    ix->names.resize(n_chrom);
    // readLine (RefReader_istr.h:48-113): case folding, other letters -> N,
    // CpGs at C - READLEN + 2 (or at C when too close to the start).
    std::vector<std::vector<fame_cpg>> cpg(n_chrom), cpgs(n_chrom);
    parallel_for(n_chrom, std::min<int>(T, (int)n_chrom), [&](uint64_t b, uint64_t e, int) {
        for (uint64_t c = b; c < e; ++c) {
            std::string& s = ix->seq[c];
            s.resize(len[c]);
            bool lastC = false;
            for (uint64_t i = 0; i < len[c]; ++i) {
                const char ch = seq[c][i];
                switch (ch) {
                    case 'g': case 'G':
                        if (lastC) {
                            if (i >= readlen - 2) cpg[c].push_back({(uint8_t)c, (uint32_t)i - readlen + 1});
                            else cpgs[c].push_back({(uint8_t)c, (uint32_t)i - 1});
                            lastC = false;
                        }
                        s[i] = 'G';
                        break;
                    case 'c': case 'C': s[i] = 'C'; lastC = true; break;
                    case 'a': case 'A': s[i] = 'A'; lastC = false; break;
                    case 't': case 'T': s[i] = 'T'; lastC = false; break;
                    default: s[i] = 'N'; lastC = false; break;
                }
            }
            ix->names[c] = names && names[c] ? std::string(names[c]) : ("chr" + std::to_string(c + 1));
        }
    });
    for (uint32_t c = 0; c < n_chrom; ++c) {
        ix->cpg.insert(ix->cpg.end(), cpg[c].begin(), cpg[c].end());
        ix->cpg_start.insert(ix->cpg_start.end(), cpgs[c].begin(), cpgs[c].end());
    }
    // generateWindows (RefGenome.cpp:532-567); cpgTable[ci] is read even at
    // ci == size there, which this treats as "no CpG".
    {
        const uint64_t ncpg = ix->cpg.size();
        uint64_t ci = 0;
        for (uint32_t c = 0; c < n_chrom; ++c) {
            for (uint32_t ws = 0; ws < ix->seq[c].size(); ws = ws + WINLEN - readlen) {
                const uint32_t we = ws + WINLEN;
                uint32_t si = CPGDUMMY, ei = CPGDUMMY;
                while (ci < ncpg && ix->cpg[ci].chrom == c && ix->cpg[ci].pos <= we) {
                    if (si == CPGDUMMY) si = (uint32_t)ci;
                    ei = (uint32_t)ci;
                    ++ci;
                }
                while (ci > 0 && ci < ncpg && ix->cpg[ci].chrom == c && ix->cpg[ci].pos >= we - readlen) --ci;
                if (ci > 0) ++ci;
                ix->win.push_back({ws, (uint8_t)c, si, ei});
            }
        }
    }
}

// filteredKmers from the k-mers in the order the reference's set received
// them, and the chromosome name order.
void fame::index_build_finish(fame_host_index* ix, std::vector<uint64_t>&& filtered_order)
{
    ix->filtered_order = std::move(filtered_order);
    ix->filtered = ix->filtered_order;
    std::sort(ix->filtered.begin(), ix->filtered.end());
    ix->filtered.erase(std::unique(ix->filtered.begin(), ix->filtered.end()), ix->filtered.end());
    ix->name_order.resize(ix->seq.size());
    for (size_t c = 0; c < ix->seq.size(); ++c) ix->name_order[c] = (uint8_t)c;   // readReference inserts in order
}

extern "C" int fame_index_build(uint32_t readlen, uint32_t n_chrom, const char* const* seq, const uint64_t* len,
                                const char* const* names, int noloss, int n_threads, fame_host_index** out)
{
    if (!out || !seq || !len || n_chrom == 0 || n_chrom > 256 || readlen <= KMERLEN || readlen >= WINLEN) return FAME_ERR_ARG;
    *out = nullptr;
    int T = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    fame_host_index* ix = new (std::nothrow) fame_host_index();
    if (!ix) return FAME_ERR_NOMEM;
    // FAME_INDEX_TIMING set: the wall time of each phase on stderr
    const bool timing = std::getenv("FAME_INDEX_TIMING") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* name) {
        if (!timing) return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "fame_index_build: %-22s %8.2f s\n", name,
                     std::chrono::duration<double>(now - t_last).count());
        t_last = now;
    };
    try {
        index_build_front(ix, readlen, n_chrom, seq, len, names, T);
        phase("sequences, CpGs, windows");
        const uint64_t nwin = ix->win.size();
        const BaseBits bb(*ix, T);
        phase("base bits");
        // pass 1: bucket sizes (estimateTablesizes)
        BigVec<uint32_t> cnt(HTABSIZE + 1);
        parallel_for(HTABSIZE + 1, T, [&](uint64_t b, uint64_t e, int) { std::memset(&cnt[b], 0, (e - b) * 4); });
        parallel_for(nwin, T, [&](uint64_t b, uint64_t e, int) {
            std::vector<uint8_t> red(WINLEN), redr(WINLEN);
            std::vector<uint32_t> iv(2 * (WINLEN + 2));
            for (uint64_t w = b; w < e; ++w)
                window_kmers(*ix, w, red.data(), redr.data(), iv.data(), [&](uint32_t key, uint32_t, int) {
                    __atomic_fetch_add(&cnt[key], 1u, __ATOMIC_RELAXED);
                });
        });
        phase("pass 1 (count)");
        // bucket starts
        uint64_t total = 0;
        {
            std::vector<uint64_t> part(T + 1, 0);
            parallel_for(HTABSIZE, T, [&](uint64_t b, uint64_t e, int t) {
                uint64_t s = 0;
                for (uint64_t i = b; i < e; ++i) s += cnt[i];
                part[t + 1] = s;
            });
            for (int t = 0; t < T; ++t) part[t + 1] += part[t];
            total = part[T];
            if (total >= 0xffffffffull) { delete ix; return FAME_ERR_INDEX; }
            ix->tab32.resize(HTABSIZE + 1);   // no zero fill: every entry is written below
            parallel_for(HTABSIZE, T, [&](uint64_t b, uint64_t e, int t) {
                uint64_t s = part[t];
                for (uint64_t i = b; i < e; ++i) { ix->tab32[i] = (uint32_t)s; s += cnt[i]; cnt[i] = (uint32_t)(s - cnt[i]); }
            });
            ix->tab32[HTABSIZE] = (uint32_t)total;
        }
        phase("bucket starts");
        // pass 2: fill with atomic cursors.  One 64-bit entry per k-mer:
        // window (bits 63-32) and its index in the window's insertion order
        // (31-16), which order the bucket, then the offset in the window
        // (15-1) and the strand (0).
        BigVec<uint64_t> ent(total);
        parallel_for(nwin, T, [&](uint64_t b, uint64_t e, int) {
            std::vector<uint8_t> red(WINLEN), redr(WINLEN);
            std::vector<uint32_t> iv(2 * (WINLEN + 2));
            for (uint64_t w = b; w < e; ++w) {
                uint32_t k = 0;
                window_kmers(*ix, w, red.data(), redr.data(), iv.data(), [&](uint32_t key, uint32_t off, int strand) {
                    const uint32_t slot = __atomic_fetch_add(&cnt[key], 1u, __ATOMIC_RELAXED);
                    ent[slot] = (w << 32) | ((uint64_t)k << 16) | ((uint64_t)off << 1) | (uint64_t)strand;
                    ++k;   // at most 2 * WINLEN k-mers per window: 16 bits
                });
            }
        });
        BigVec<uint32_t>().swap(cnt);
        phase("pass 2 (fill)");
        // per bucket: reverse insertion order, then the two filters.  keep[i]
        // marks survivors; filtered k-mer sequences are collected per thread.
        BigVec<uint8_t> keep(total);
        std::vector<std::vector<uint64_t>> filt(T);
        std::vector<uint64_t> kept_in(T + 1, 0);   // survivors per thread range (the compaction's partition)
        parallel_for(HTABSIZE, T, [&](uint64_t b, uint64_t e, int t) {
            std::vector<uint64_t> ks, sorted, seen;
            std::vector<uint32_t> masks;
            uint64_t kept_sum = 0;
            for (uint64_t key = b; key < e; ++key) {
                const uint32_t s0 = ix->tab32[key], s1 = ix->tab32[key + 1];
                const uint32_t n = s1 - s0;
                if (n == 0) continue;
                uint64_t* E = &ent[s0];
                if (n > 1) std::sort(E, E + n, std::greater<uint64_t>());   // reverse insertion order
                std::memset(&keep[s0], 1, n);
                // filterHashTable (RefGenome.cpp:2267-2352)
                if (!noloss && n >= KMERCUTOFF) {
                    ks.resize(n); sorted.resize(n);
                    for (uint32_t i = 0; i < n; ++i)
                        ks[i] = sorted[i] = kmer_seq(*ix, ent_win(E[i]), ent_off(E[i]), ent_fwd(E[i]));
                    std::sort(sorted.begin(), sorted.end());
                    seen.clear();
                    for (uint32_t i = 0; i < n; ++i) {
                        auto r = std::equal_range(sorted.begin(), sorted.end(), ks[i]);
                        if ((uint64_t)(r.second - r.first) >= KMERCUTOFF) {
                            keep[s0 + i] = 0;
                            // the set's insertion order (RefGenome.cpp:2330): first occurrence in bucket order
                            if (std::find(seen.begin(), seen.end(), ks[i]) == seen.end()) {
                                seen.push_back(ks[i]);
                                filt[t].push_back(ks[i]);
                            }
                        }
                    }
                }
                // filterRedundancyInHashTable (RefGenome.cpp:2191-2264)
                uint64_t prevMeta = ~0ull;
                int prevFwd = 0;
                masks.clear();
                uint32_t kept = 0;
                for (uint32_t i = 0; i < n; ++i) {
                    if (!keep[s0 + i]) continue;
                    const uint32_t w = ent_win(E[i]);
                    const int fwd = ent_fwd(E[i]);
                    const uint32_t tm = tmask_repro(*ix, bb, w, ent_off(E[i]), fwd);
                    if (w != prevMeta || fwd != prevFwd) {
                        masks.clear();
                        masks.push_back(tm);
                        prevMeta = w;
                        prevFwd = fwd;
                        ++kept;
                    } else if (std::find(masks.begin(), masks.end(), tm) == masks.end()) {
                        masks.push_back(tm);
                        ++kept;
                    } else {
                        keep[s0 + i] = 0;
                    }
                }
                kept_sum += kept;
            }
            kept_in[t + 1] = kept_sum;
        });
        phase("bucket order, filters");
        // compaction
        uint64_t nk = 0;
        {
            std::vector<uint64_t> part(kept_in);
            for (int t = 0; t < T; ++t) part[t + 1] += part[t];
            nk = part[T];
            ix->kmer.resize(nk);
            BigVec<uint8_t> kstr(nk);     // every entry written below
            BigVec<uint32_t> koff(nk);
            // the old start of each thread's first key after its range, read
            // before any thread rewrites tab32 (same partition as parallel_for)
            std::vector<uint32_t> bound(T, 0);
            {
                const uint64_t step = (HTABSIZE + T - 1) / T;
                for (int t = 0; t < T; ++t) bound[t] = ix->tab32[std::min<uint64_t>(HTABSIZE, (uint64_t)t * step + step)];
            }
            parallel_for(HTABSIZE, T, [&](uint64_t b, uint64_t e, int t) {
                uint64_t o = part[t];
                for (uint64_t key = b; key < e; ++key) {
                    const uint32_t s0 = ix->tab32[key], s1 = key + 1 == e ? bound[t] : ix->tab32[key + 1];
                    ix->tab32[key] = (uint32_t)o;
                    for (uint32_t i = s0; i < s1; ++i) {
                        if (!keep[i]) continue;
                        ix->kmer[o].meta = ent_win(ent[i]);
                        kstr[o] = (uint8_t)ent_fwd(ent[i]);
                        koff[o] = ent_off(ent[i]);
                        ++o;
                    }
                }
            });
            ix->tab32[HTABSIZE] = (uint32_t)nk;
            phase("compaction");
            // strandTable
            ix->strand_bits.resize((nk + 7) / 8);
            parallel_for((nk + 7) / 8, T, [&](uint64_t b, uint64_t e, int) {
                for (uint64_t j = b; j < e; ++j) {
                    uint8_t v = 0;
                    for (uint64_t i = 8 * j; i < std::min<uint64_t>(8 * j + 8, nk); ++i)
                        if (kstr[i]) v |= (uint8_t)(1u << (i & 7));
                    ix->strand_bits[j] = v;
                }
            });
            phase("strand bits");
            // getTMask at save time (RefGenome.h:62-100): strand taken at
            // strandTable[window id]; the reverse loop skips base 0.
            parallel_for(nk, T, [&](uint64_t b, uint64_t e, int) {
                for (uint64_t k = b; k < e; ++k) {
                    const uint32_t w = ix->kmer[k].meta & 0x7fffffffu;
                    const uint32_t c = ix->win[w].chrom;
                    const uint64_t s0 = (uint64_t)ix->win[w].start_pos + koff[k];
                    const int fwd = w < nk ? kstr[w] : 0;
                    // forward: bit 31 - i is 'T' at s0 + i; reverse (i = 31 .. 1):
                    // bit i - 1 is 'A' at s0 + i, bit 31 stays 0
                    const uint32_t tm = fwd ? bb.t_fwd(c, s0) : (bb.a_lo(c, s0 + 1) & 0x7fffffffu);
                    ix->kmer[k].tmask = tm;
                }
            });
        }
        phase("T masks");
        // threads hold consecutive bucket ranges: their lists in thread order are the scan order
        std::vector<uint64_t> order;
        for (auto& f : filt) order.insert(order.end(), f.begin(), f.end());
        index_build_finish(ix, std::move(order));
        phase("filtered set");
    } catch (const std::bad_alloc&) {
        delete ix;
        return FAME_ERR_NOMEM;
    } catch (const std::exception&) {   // a worker thread's failure, rethrown by parallel_for
        delete ix;
        return FAME_ERR_NOMEM;
    }
    *out = ix;
    return FAME_OK;
}

// ---------------------------------------------------------------------------
// --load_index reader (RefGenome.cpp:230-433)
// ---------------------------------------------------------------------------
namespace {
struct Reader {
    FILE* f;
    bool ok = true;
    template <class T> T get() { T v{}; if (fread(&v, sizeof(T), 1, f) != 1) ok = false; return v; }
    void bytes(void* p, uint64_t n) { if (n && fread(p, 1, n, f) != n) ok = false; }
};
}  // namespace

extern "C" int fame_index_read(const char* path, fame_host_index** out)
{
    if (!path || !out) return FAME_ERR_ARG;
    *out = nullptr;
    FILE* f = fopen(path, "rb");
    if (!f) return FAME_ERR_IO;
    fame_host_index* ix = new (std::nothrow) fame_host_index();
    if (!ix) { fclose(f); return FAME_ERR_NOMEM; }
    Reader r{f};
    int rc = FAME_OK;
    try {
        const uint64_t htabs = r.get<uint64_t>();
        const uint32_t readl = r.get<uint32_t>(), winl = r.get<uint32_t>(), kmerl = r.get<uint32_t>();
        const uint64_t kmerc = r.get<uint64_t>();
        const uint32_t seedbits = r.get<uint32_t>();
        if (!r.ok || htabs != HTABSIZE || winl != WINLEN || kmerl != KMERLEN || kmerc != KMERCUTOFF ||
            seedbits != SEEDBITS || readl <= KMERLEN || readl >= WINLEN) {
            rc = FAME_ERR_IO;
        } else {
            ix->readlen = readl;
            uint64_t n = r.get<uint64_t>();
            ix->cpg.resize(n); r.bytes(ix->cpg.data(), n * sizeof(fame_cpg));
            n = r.get<uint64_t>();
            ix->cpg_start.resize(n); r.bytes(ix->cpg_start.data(), n * sizeof(fame_cpg));
            n = r.get<uint64_t>();
            if (n > 256) throw std::bad_alloc();
            ix->seq.resize(n);
            for (auto& s : ix->seq) { uint64_t l = r.get<uint64_t>(); s.resize(l); r.bytes(&s[0], l); }
            n = r.get<uint64_t>();
            if (n != HTABSIZE + 1) throw std::length_error("tabIndex size");
            ix->tab64.resize(n);
            {
                // the 8 GiB table: read by several threads at their own offsets
                const off_t at = ftello(f);
                const uint64_t bytes = n * 8;
                const int T = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
                std::atomic<bool> good{at >= 0};
                char* dst = reinterpret_cast<char*>(ix->tab64.data());
                if (at < 0) {
                    r.bytes(dst, bytes);   // not seekable (a pipe): read in order through the stream
                } else {
                    parallel_for(bytes, T, [&](uint64_t b, uint64_t e, int) {
                        while (b < e && good.load(std::memory_order_relaxed)) {
                            const ssize_t got = pread(fileno(f), dst + b,
                                                      (size_t)std::min<uint64_t>(e - b, 1ull << 30), at + (off_t)b);
                            if (got <= 0) { good = false; break; }
                            b += (uint64_t)got;
                        }
                    });
                    if (!good || fseeko(f, at + (off_t)bytes, SEEK_SET) != 0) r.ok = false;
                }
            }
            n = r.get<uint64_t>();
            ix->kmer.resize(n); r.bytes(ix->kmer.data(), n * sizeof(fame_kmer));
            uint64_t m = r.get<uint64_t>();      // metaCpGs (unused by the window index)
            fseek(f, (long)(m * 8), SEEK_CUR);
            m = r.get<uint64_t>();               // metaStartCpGs
            fseek(f, (long)(m * 8), SEEK_CUR);
            n = r.get<uint64_t>();
            ix->win.resize(n); r.bytes(ix->win.data(), n * sizeof(fame_window));
            n = r.get<uint64_t>();
            ix->filtered_order.resize(n); r.bytes(ix->filtered_order.data(), n * 8);
            ix->filtered = ix->filtered_order;
            std::sort(ix->filtered.begin(), ix->filtered.end());
            n = r.get<uint64_t>();
            ix->names.assign(ix->seq.size(), std::string());
            for (uint64_t i = 0; i < n && r.ok; ++i) {
                const uint8_t id = r.get<uint8_t>();
                const uint64_t l = r.get<uint64_t>();
                std::string s(l, '\0');
                r.bytes(&s[0], l);
                if (id < ix->names.size()) ix->names[id] = s;
                ix->name_order.push_back(id);
            }
            if (!r.ok || ix->tab64.size() != HTABSIZE + 1 || ix->tab64.back() != ix->kmer.size()) rc = FAME_ERR_IO;
        }
    } catch (const std::bad_alloc&) {
        rc = FAME_ERR_NOMEM;
    } catch (const std::exception&) {   // a size field no index file can hold
        rc = FAME_ERR_IO;
    }
    fclose(f);
    if (rc == FAME_OK) {
        const std::string sp = std::string(path) + "_strands";
        FILE* g = fopen(sp.c_str(), "rb");
        if (!g) rc = FAME_ERR_IO;
        else {
            Reader rs{g};
            const uint64_t n = rs.get<uint64_t>();
            ix->strand_bits.resize((n + 7) / 8);
            rs.bytes(ix->strand_bits.data(), ix->strand_bits.size());
            if (!rs.ok || n != ix->kmer.size()) rc = FAME_ERR_IO;
            fclose(g);
        }
    }
    if (rc != FAME_OK) { delete ix; return rc; }
    *out = ix;
    return FAME_OK;
}

// ---------------------------------------------------------------------------
// --load_index writer (RefGenome::save, RefGenome.cpp:83-228; write_strands
// 392-413; write_filteredKmers 434-443)
// ---------------------------------------------------------------------------
namespace {

struct Writer {
    FILE* f;
    bool ok = true;
    template <class T> void put(T v) { if (fwrite(&v, sizeof(T), 1, f) != 1) ok = false; }
    void bytes(const void* p, uint64_t n) { if (n && fwrite(p, 1, n, f) != n) ok = false; }
};

// The reference's KmerHash (RefGenome.h:215-222): the k-mer itself.
struct KmerIdentity {
    size_t operator()(const uint64_t& k) const { return static_cast<size_t>(k); }
};

// Structs written as the reference writes them (raw, 8 and 16 bytes); the
// padding bytes, uninitialised there, are zero here.
void put_cpgs(Writer& w, const std::vector<fame_cpg>& v)
{
    w.put<uint64_t>(v.size());
    std::vector<uint8_t> blk;
    for (size_t i = 0; i < v.size(); i += 65536) {
        const size_t n = std::min<size_t>(65536, v.size() - i);
        blk.assign(n * 8, 0);
        for (size_t j = 0; j < n; ++j) {
            blk[8 * j] = v[i + j].chrom;
            std::memcpy(&blk[8 * j + 4], &v[i + j].pos, 4);
        }
        w.bytes(blk.data(), blk.size());
    }
}

}  // namespace

extern "C" int fame_index_write(const fame_host_index* ix, const char* path)
{
    if (!ix || !path || (ix->tab32.empty() && ix->tab64.empty())) return FAME_ERR_ARG;
    FILE* f = fopen(path, "wb");
    if (!f) return FAME_ERR_IO;
    std::vector<char> vbuf(8u << 20);
    setvbuf(f, vbuf.data(), _IOFBF, vbuf.size());
    Writer w{f};
    try {
        w.put<uint64_t>(HTABSIZE);
        w.put<uint32_t>(ix->readlen);
        w.put<uint32_t>(WINLEN);
        w.put<uint32_t>(KMERLEN);
        w.put<uint64_t>(KMERCUTOFF);
        w.put<uint32_t>(SEEDBITS);
        put_cpgs(w, ix->cpg);
        put_cpgs(w, ix->cpg_start);
        w.put<uint64_t>(ix->seq.size());
        for (const auto& s : ix->seq) {
            w.put<uint64_t>(s.size());
            w.bytes(s.data(), s.size());
        }
        // tabIndex as uint64
        w.put<uint64_t>(HTABSIZE + 1);
        {
            // the 8 GiB table: written by several threads at their own offsets
            const off_t at = (fflush(f) == 0) ? ftello(f) : (off_t)-1;
            const uint64_t n = HTABSIZE + 1;
            const int T = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
            std::atomic<bool> good{at >= 0};
            constexpr uint64_t BLK = 1u << 20;
            if (at < 0) {
                // not seekable (a pipe): written in order through the stream
                std::vector<uint64_t> blk(ix->tab64.empty() ? BLK : 0);
                for (uint64_t i = 0; i < n && w.ok; i += BLK) {
                    const uint64_t m = std::min<uint64_t>(BLK, n - i);
                    const uint64_t* src = ix->tab64.empty() ? blk.data() : ix->tab64.data() + i;
                    if (ix->tab64.empty())
                        for (uint64_t j = 0; j < m; ++j) blk[j] = ix->tab32[i + j];
                    w.bytes(src, m * 8);
                }
            } else {
                parallel_for(n, T, [&](uint64_t b, uint64_t e, int) {
                    // a conversion block only when the offsets are held as uint32
                    std::vector<uint64_t> blk(ix->tab64.empty() ? BLK : 0);
                    for (uint64_t i = b; i < e && good.load(std::memory_order_relaxed); i += BLK) {
                        const uint64_t m = std::min<uint64_t>(BLK, e - i);
                        const uint64_t* src = ix->tab64.empty() ? blk.data() : ix->tab64.data() + i;
                        if (ix->tab64.empty())
                            for (uint64_t j = 0; j < m; ++j) blk[j] = ix->tab32[i + j];
                        const char* p = reinterpret_cast<const char*>(src);
                        uint64_t left = m * 8, done = 0;
                        while (left) {
                            const ssize_t put = pwrite(fileno(f), p + done, (size_t)left, at + (off_t)(8 * i + done));
                            if (put <= 0) { good = false; break; }
                            done += (uint64_t)put;
                            left -= (uint64_t)put;
                        }
                    }
                });
                if (!good || fseeko(f, at + (off_t)(n * 8), SEEK_SET) != 0) w.ok = false;
            }
        }
        // k-mers: KMER::getCore and the T mask of each (the loaded layout)
        w.put<uint64_t>(ix->kmer.size());
        w.bytes(ix->kmer.data(), ix->kmer.size() * sizeof(fame_kmer));
        w.put<uint64_t>(0);   // metaCpGs: empty in the window index
        w.put<uint64_t>(0);   // metaStartCpGs
        w.put<uint64_t>(ix->win.size());
        {
            std::vector<uint8_t> blk;
            for (size_t i = 0; i < ix->win.size(); i += 65536) {
                const size_t n = std::min<size_t>(65536, ix->win.size() - i);
                blk.assign(n * 16, 0);
                for (size_t j = 0; j < n; ++j) {
                    const fame_window& x = ix->win[i + j];
                    std::memcpy(&blk[16 * j], &x.start_pos, 4);
                    blk[16 * j + 4] = x.chrom;
                    std::memcpy(&blk[16 * j + 8], &x.start_ind, 4);
                    std::memcpy(&blk[16 * j + 12], &x.end_ind, 4);
                }
                w.bytes(blk.data(), blk.size());
            }
        }
        // filteredKmers and chrMap in the iteration order of the reference's
        // unordered containers: the same container types receiving the same
        // keys in the same order iterate the same way
        {
            std::unordered_set<uint64_t, KmerIdentity> fk;
            for (uint64_t k : ix->filtered_order) fk.emplace(k);
            w.put<uint64_t>(fk.size());
            for (uint64_t k : fk) w.put<uint64_t>(k);
        }
        {
            std::unordered_map<uint8_t, std::string> cm;
            for (uint8_t id : ix->name_order)
                if (id < ix->names.size()) cm.insert(std::pair<uint8_t, std::string>(id, ix->names[id]));
            w.put<uint64_t>(cm.size());
            for (const auto& e : cm) {
                w.put<uint8_t>(e.first);
                w.put<uint64_t>(e.second.size());
                w.bytes(e.second.data(), e.second.size());
            }
        }
    } catch (const std::bad_alloc&) {
        fclose(f);
        return FAME_ERR_NOMEM;
    } catch (const std::exception&) {
        fclose(f);
        return FAME_ERR_IO;
    }
    if (fclose(f) != 0) w.ok = false;
    if (!w.ok) return FAME_ERR_IO;
    // <path>_strands: k-mer count, then the strand bits LSB first
    FILE* g = fopen((std::string(path) + "_strands").c_str(), "wb");
    if (!g) return FAME_ERR_IO;
    Writer ws{g};
    ws.put<uint64_t>(ix->kmer.size());
    ws.bytes(ix->strand_bits.data(), (ix->kmer.size() + 7) / 8);
    if (fclose(g) != 0) ws.ok = false;
    return ws.ok ? FAME_OK : FAME_ERR_IO;
}

extern "C" int fame_index_view_of(const fame_host_index* cix, fame_index_view* v)
{
    if (!cix || !v) return FAME_ERR_ARG;
    fame_host_index* ix = const_cast<fame_host_index*>(cix);
    ix->seq_ptrs.resize(ix->seq.size());
    ix->seq_lens.resize(ix->seq.size());
    ix->name_ptrs.resize(ix->seq.size());
    if (ix->names.size() < ix->seq.size()) ix->names.resize(ix->seq.size());
    for (size_t c = 0; c < ix->seq.size(); ++c) {
        ix->seq_ptrs[c] = ix->seq[c].data();
        ix->seq_lens[c] = ix->seq[c].size();
        ix->name_ptrs[c] = ix->names[c].c_str();
    }
    memset(v, 0, sizeof(*v));
    v->readlen = ix->readlen;
    v->n_chrom = (uint32_t)ix->seq.size();
    v->chrom_seq = ix->seq_ptrs.data();
    v->chrom_len = ix->seq_lens.data();
    v->chrom_name = ix->name_ptrs.data();
    v->n_cpg = ix->cpg.size();
    v->cpg = ix->cpg.data();
    v->tab_index = ix->tab64.empty() ? nullptr : ix->tab64.data();
    v->tab_index32 = ix->tab32.empty() ? nullptr : ix->tab32.data();
    v->n_kmer = ix->kmer.size();
    v->kmer = ix->kmer.data();
    v->strand_bits = ix->strand_bits.data();
    v->n_win = ix->win.size();
    v->win = ix->win.data();
    v->n_filtered = ix->filtered.size();
    v->filtered = ix->filtered.data();
    return FAME_OK;
}

extern "C" void fame_index_free(fame_host_index* ix) { delete ix; }

// Start CpGs (never reported, RefReader_istr.h:66-76) for the index file writer and tests.
extern "C" uint64_t fame_index_cpg_start(const fame_host_index* ix, fame_cpg* out, uint64_t cap)
{
    if (!ix) return 0;
    for (uint64_t i = 0; i < ix->cpg_start.size() && i < cap; ++i) out[i] = ix->cpg_start[i];
    return ix->cpg_start.size();
}

extern "C" uint64_t fame_index_filtered_order(const fame_host_index* ix, uint64_t* out, uint64_t cap)
{
    if (!ix) return 0;
    for (uint64_t i = 0; i < ix->filtered_order.size() && i < cap; ++i) out[i] = ix->filtered_order[i];
    return ix->filtered_order.size();
}
