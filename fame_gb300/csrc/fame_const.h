// Compile-time parameters of FAME's matching path (CONST.h:35-110).  The
// device kernels and the host index code are built for exactly these values;
// an index file written with others is rejected on open.
#pragma once
#include <stdint.h>

namespace fame {

constexpr uint64_t HTABSIZE = 1ull << 30;          // CONST.h:85
constexpr uint32_t HTAB_MASK = (1u << 30) - 1;
constexpr uint32_t KMERLEN = 32;                    // CONST.h:73
constexpr uint32_t SEEDBITS = 0xDEFDFFFDu;          // CONST.h:58 (bit 31 = seed position 0)
constexpr uint32_t WINLEN = 2048;                   // CONST.h:90
constexpr uint32_t MISCOUNT = 2;                    // CONST.h:94
constexpr uint32_t ADDMIS = 4;                      // CONST.h:97
constexpr uint32_t NERR = MISCOUNT + ADDMIS;        // ShiftAnd<MISCOUNT + ADDMIS>
constexpr uint32_t QTHRESH = 5;                     // CONST.h:80
constexpr uint64_t KMERCUTOFF = 1500;               // CONST.h:101
constexpr uint32_t SKIPMOD = 2;                     // CONST.h:107
constexpr uint32_t CPGDUMMY = 0xffffffffu;          // CONST.h:110
constexpr uint32_t CHUNKSIZE = 300000;              // CONST.h:69
constexpr uint32_t DP_BAND = 2 * MISCOUNT + ADDMIS; // LevenshtDP<uint16_t, 8> (ReadQueue.cpp:3626)
constexpr uint32_t WIN_TEXT = WINLEN + MISCOUNT + ADDMIS - 1; // window text scanned (ReadQueue.cpp:1955)

// spaced_nthash/nthash.hpp:20-26: per-base 64-bit seeds; the reduced alphabet
// hashes C with the T seed (msTab, nthash.hpp:88-121).
constexpr uint64_t NT_SEED_A = 0x3c8bfbb395c60474ULL;
constexpr uint64_t NT_SEED_G = 0x20323ed082572324ULL;
constexpr uint64_t NT_SEED_T = 0x295549f54be24456ULL;

}  // namespace fame
