// Spaced-seed k-mer hash of the seeding stage (NTPS64 of spaced_nthash, the
// reduced alphabet of getSeedRefs: C hashes with the T seed), host and device.
//
// The hash of the 32-base k-mer at read position p is
//     H(p) = XOR over the seed's care positions i of rotl(v[p + i], 31 - i),
// v[j] the msTab value of read base j (nthash.hpp:88-121; the rolling NTPS64
// update equals this direct form).  With u[j] = rotr(v[j], j mod 64) every
// care term is rotl(u[p + i], p + 31), so
//     H(p) = rotl(P[p + 32] ^ P[p] ^ XOR over don't-care i of u[p + i], p + 31)
// where P[j] = u[0] ^ ... ^ u[j - 1] is a prefix XOR over the read: a warp
// builds P once per read and each k-mer then costs a few loads instead of 28
// rotate-and-XOR terms.
#pragma once
#include <stdint.h>

#include "fame_const.h"

#if defined(__CUDACC__)
#define FAME_HD __host__ __device__ __forceinline__
#else
#define FAME_HD inline
#endif

namespace fame {

FAME_HD uint64_t sh_rotl(uint64_t v, unsigned s)
{
    s &= 63u;
    return s ? (v << s) | (v >> (64 - s)) : v;
}

FAME_HD uint64_t sh_rotr(uint64_t v, unsigned s)
{
    s &= 63u;
    return s ? (v >> s) | (v << (64 - s)) : v;
}

// msTab value of a read byte (spaced_nthash/nthash.hpp:88-121)
FAME_HD uint64_t sh_nt(uint8_t c)
{
    switch (c) {
        case 'A': case 'a': case 4: return NT_SEED_A;
        case 'C': case 'c': case 'T': case 't': case 1: case 7: return NT_SEED_T;
        case 'G': case 'g': case 3: return NT_SEED_G;
        default: return 0;
    }
}

// The direct form over the care positions.
FAME_HD uint64_t sh_direct(const uint8_t* seq, uint32_t p)
{
    uint64_t h = 0;
    for (uint32_t i = 0; i < KMERLEN; ++i)
        if ((SEEDBITS >> (31 - i)) & 1u) h ^= sh_rotl(sh_nt(seq[p + i]), 31 - i);
    return h;
}

// u[j] of the prefix form.
FAME_HD uint64_t sh_u(uint8_t c, uint32_t j) { return sh_rotr(sh_nt(c), j); }

// Low 32 bits of rotl(x, r).
FAME_HD uint32_t sh_rotl_lo32(uint64_t x, unsigned r)
{
    r &= 63u;
    const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
    const uint32_t a = r < 32 ? hi : lo, b = r < 32 ? lo : hi;   // rotl(x, r) low word = (b:a) << (r mod 32), upper half
    const unsigned s = r & 31u;
    return s ? (b << s) | (a >> (32 - s)) : b;
}

// H(p) & mask from the prefix array (P[0 .. p + 32] read).
template <class Load>
FAME_HD uint32_t sh_prefix_hash(Load P, uint32_t p, uint32_t mask)
{
    uint64_t x = P(p + KMERLEN) ^ P(p);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (uint32_t i = 0; i < KMERLEN; ++i)
        if (!((SEEDBITS >> (31 - i)) & 1u)) x ^= P(p + i + 1) ^ P(p + i);
    return sh_rotl_lo32(x, p + 31) & mask;
}

}  // namespace fame
