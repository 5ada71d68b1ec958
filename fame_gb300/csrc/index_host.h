// Host-side index tables (the loaded RefGenome members, RefGenome.h:193-227).
#pragma once
#include <stdint.h>
#include <sys/mman.h>

#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fame_gpu.h"

// An allocator for the multi-GiB tables that the builder fills in parallel
// anyway: value-initialisation leaves the storage unset, and blocks of 64 MiB
// or more are mapped directly with transparent huge pages requested, so the
// threads that first write them take a few large page faults, not millions.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    static constexpr size_t kMapped = size_t(64) << 20;
    template <class U> struct rebind { using other = NoInitAlloc<U>; };
    NoInitAlloc() = default;
    template <class U> NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    T* allocate(size_t n)
    {
        const size_t bytes = n * sizeof(T);
        if (bytes < kMapped) return std::allocator<T>::allocate(n);
        void* p = ::mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
        if (p == MAP_FAILED) throw std::bad_alloc();
        ::madvise(p, bytes, MADV_HUGEPAGE);
        return static_cast<T*>(p);
    }
    void deallocate(T* p, size_t n) noexcept
    {
        const size_t bytes = n * sizeof(T);
        if (bytes < kMapped) std::allocator<T>::deallocate(p, n);
        else ::munmap(p, bytes);
    }
    template <class U> void construct(U* p) noexcept { ::new ((void*)p) U; }
    template <class U, class... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};
template <class T, class U> bool operator==(const NoInitAlloc<T>&, const NoInitAlloc<U>&) { return true; }
template <class T, class U> bool operator!=(const NoInitAlloc<T>&, const NoInitAlloc<U>&) { return false; }
template <class T> using BigVec = std::vector<T, NoInitAlloc<T>>;

struct fame_host_index {
    uint32_t readlen = 0;
    std::vector<std::string> seq;        // fullSeq: ACGTN
    std::vector<std::string> names;      // chrMap
    std::vector<fame_cpg> cpg;           // cpgTable
    std::vector<fame_cpg> cpg_start;     // cpgStartTable
    BigVec<uint32_t> tab32;              // tabIndex as uint32 (HTABSIZE + 1)
    BigVec<uint64_t> tab64;              // or as read from a file (uint64)
    BigVec<fame_kmer> kmer;              // kmerTableSmall
    std::vector<uint8_t> strand_bits;    // strandTable, LSB first
    std::vector<fame_window> win;        // metaWindows
    std::vector<uint64_t> filtered;      // filteredKmers (sorted)
    std::vector<uint64_t> filtered_order;  // the same k-mers in the order the reference's set received them
    std::vector<uint8_t> name_order;     // chrMap ids in the order the reference's map received them
    std::vector<const char*> seq_ptrs;   // for views
    std::vector<uint64_t> seq_lens;
    std::vector<const char*> name_ptrs;
};

namespace fame {
// readReference and generateWindows (RefReader_istr.h:48-113,
// RefGenome.cpp:532-567): fills seq, names, cpg, cpg_start and win on T
// host threads.
void index_build_front(fame_host_index* ix, uint32_t readlen, uint32_t n_chrom, const char* const* seq,
                       const uint64_t* len, const char* const* names, int T);
// filtered_order as given, filtered (sorted, unique) and name_order.
void index_build_finish(fame_host_index* ix, std::vector<uint64_t>&& filtered_order);
}  // namespace fame
