// Host-side index tables (the loaded RefGenome members, RefGenome.h:193-227).
#pragma once
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/fame_gpu.h"

struct fame_host_index {
    uint32_t readlen = 0;
    std::vector<std::string> seq;        // fullSeq: ACGTN
    std::vector<std::string> names;      // chrMap
    std::vector<fame_cpg> cpg;           // cpgTable
    std::vector<fame_cpg> cpg_start;     // cpgStartTable
    std::vector<uint32_t> tab32;         // tabIndex as uint32 (HTABSIZE + 1)
    std::vector<uint64_t> tab64;         // or as read from a file (uint64)
    std::vector<fame_kmer> kmer;         // kmerTableSmall
    std::vector<uint8_t> strand_bits;    // strandTable, LSB first
    std::vector<fame_window> win;        // metaWindows
    std::vector<uint64_t> filtered;      // filteredKmers (sorted)
    std::vector<uint64_t> filtered_order;  // the same k-mers in the order the reference's set received them
    std::vector<uint8_t> name_order;     // chrMap ids in the order the reference's map received them
    std::vector<const char*> seq_ptrs;   // for views
    std::vector<uint64_t> seq_lens;
    std::vector<const char*> name_ptrs;
};
