// Host-side index tables (the loaded RefGenome members, RefGenome.h:193-227).
#pragma once
#include <stdint.h>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fame_gpu.h"

// An allocator whose value-initialisation leaves the storage unset, for the
// multi-GiB tables that the builder fills in parallel anyway.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = NoInitAlloc<U>; };
    NoInitAlloc() = default;
    template <class U> NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U> void construct(U* p) noexcept { ::new ((void*)p) U; }
    template <class U, class... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};

struct fame_host_index {
    uint32_t readlen = 0;
    std::vector<std::string> seq;        // fullSeq: ACGTN
    std::vector<std::string> names;      // chrMap
    std::vector<fame_cpg> cpg;           // cpgTable
    std::vector<fame_cpg> cpg_start;     // cpgStartTable
    std::vector<uint32_t, NoInitAlloc<uint32_t>> tab32;   // tabIndex as uint32 (HTABSIZE + 1)
    std::vector<uint64_t> tab64;         // or as read from a file (uint64)
    std::vector<fame_kmer, NoInitAlloc<fame_kmer>> kmer;  // kmerTableSmall
    std::vector<uint8_t> strand_bits;    // strandTable, LSB first
    std::vector<fame_window> win;        // metaWindows
    std::vector<uint64_t> filtered;      // filteredKmers (sorted)
    std::vector<uint64_t> filtered_order;  // the same k-mers in the order the reference's set received them
    std::vector<uint8_t> name_order;     // chrMap ids in the order the reference's map received them
    std::vector<const char*> seq_ptrs;   // for views
    std::vector<uint64_t> seq_lens;
    std::vector<const char*> name_ptrs;
};
