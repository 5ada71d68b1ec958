// DEFLATE decoder (RFC 1951) for one raw stream with a known output size, and
// CRC-32 (the gzip member trailer's checksum, RFC 1952), for the host and the
// device: the device inflates BGZF input (gzip members of at most 64 KiB, the
// layout bgzip writes) one member per thread; the host copy is what the
// native checks run against zlib.
//
// Written from the format's description: canonical Huffman codes decoded
// through a 9-bit lookup table (the bit-reversed codes of up to 9 bits, each
// filling every entry it prefixes), longer codes a bit at a time (codes of one
// length are consecutive integers, so a code of length L is valid when
// code - first[L] < count[L]); stored, fixed-code and dynamic-code blocks;
// the length and distance base tables of RFC 1951 §3.2.5.  The code tables
// live in a scratch the caller provides (on the device, shared memory of the
// warp whose lanes all run the same member in step).  Every input read, output write and back-reference is checked
// against its bounds; malformed input gives an error code, never an access
// outside the buffers.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define FAME_HD __host__ __device__
#else
#define FAME_HD
#endif

namespace fame {

enum {
    INFL_OK = 0,
    INFL_ERR_INPUT = 1,     // the stream ends early
    INFL_ERR_BLOCK = 2,     // block type 3, or a stored block's length check fails
    INFL_ERR_CODE = 3,      // over-subscribed code lengths, or a code not in the table
    INFL_ERR_DIST = 4,      // a back-reference before the start of the output
    INFL_ERR_SIZE = 5,      // more output than the declared size, or less at the end
    INFL_ERR_CRC = 6,       // CRC-32 of the output differs from the trailer
    INFL_ERR_HEADER = 7,    // not a BGZF member
};

struct InflBits {
    const uint8_t* in;
    uint32_t len, pos;
    uint64_t buf;   // bits not yet used, least significant first
    uint32_t cnt;
};

FAME_HD inline bool infl_need(InflBits& b, uint32_t n)
{
    while (b.cnt < n) {
        if (b.pos >= b.len) return false;
        b.buf |= (uint64_t)b.in[b.pos++] << b.cnt;
        b.cnt += 8;
    }
    return true;
}

// n <= 32 bits, least significant bit first
FAME_HD inline bool infl_bits(InflBits& b, uint32_t n, uint32_t& v)
{
    if (!infl_need(b, n)) return false;
    v = (uint32_t)(b.buf & ((n == 32) ? 0xffffffffull : ((1ull << n) - 1)));
    b.buf >>= n;
    b.cnt -= n;
    return true;
}

// A canonical code: how many codes of each length 1..15, the symbols in code
// order (by length, then symbol value), and for codes of up to INFL_FAST
// bits a table indexed by the next INFL_FAST input bits: symbol << 4 | code
// length, 0 where no such code starts.
constexpr uint32_t INFL_FAST = 9;
struct InflCode {
    uint16_t count[16];
    uint16_t sym[288];
    uint16_t fast[1u << INFL_FAST];
};

struct InflScratch {
    InflCode lit, dist;
    uint8_t lens[320];
};

// Returns false for over-subscribed lengths; incomplete codes are allowed
// (a code outside them fails when decoded).
FAME_HD inline bool infl_build(InflCode& c, const uint8_t* lens, uint32_t n)
{
    for (int l = 0; l < 16; ++l) c.count[l] = 0;
    for (uint32_t s = 0; s < n; ++s) c.count[lens[s]]++;
    c.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left = 2 * left - c.count[l];
        if (left < 0) return false;
    }
    uint16_t start[16], next[16];
    start[1] = 0;
    for (int l = 1; l < 15; ++l) start[l + 1] = (uint16_t)(start[l] + c.count[l]);
    // first code of each length (RFC 1951 §3.2.2)
    uint32_t code = 0;
    next[0] = 0;
    for (int l = 1; l < 16; ++l) {
        code = (code + c.count[l - 1]) << 1;
        next[l] = (uint16_t)code;
    }
    for (uint32_t i = 0; i < (1u << INFL_FAST); ++i) c.fast[i] = 0;
    for (uint32_t s = 0; s < n; ++s) {
        const uint32_t l = lens[s];
        if (!l) continue;
        c.sym[start[l]++] = (uint16_t)s;
        const uint32_t cd = next[l]++;
        if (l <= INFL_FAST) {
            uint32_t rev = 0;   // the stream holds the code's most significant bit first
            for (uint32_t k = 0; k < l; ++k) rev |= ((cd >> k) & 1u) << (l - 1 - k);
            for (uint32_t i = rev; i < (1u << INFL_FAST); i += 1u << l) c.fast[i] = (uint16_t)(s << 4 | l);
        }
    }
    return true;
}

// The next symbol, or -1 when the stream ends or the code is not assigned.
FAME_HD inline int infl_decode(InflBits& b, const InflCode& c)
{
    while (b.cnt < INFL_FAST && b.pos < b.len) {   // as many of the next bits as there are
        b.buf |= (uint64_t)b.in[b.pos++] << b.cnt;
        b.cnt += 8;
    }
    const uint32_t e = c.fast[b.buf & ((1u << INFL_FAST) - 1)];
    if (e && (e & 15u) <= b.cnt) {
        b.buf >>= (e & 15u);
        b.cnt -= (e & 15u);
        return (int)(e >> 4);
    }
    uint32_t code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        if (!infl_need(b, 1)) return -1;
        code |= (uint32_t)(b.buf & 1u);   // Huffman codes are packed most significant bit first
        b.buf >>= 1;
        b.cnt -= 1;
        const uint32_t cnt = c.count[l];
        if (code - first < cnt) return c.sym[index + code - first];
        index += cnt;
        first = (first + cnt) << 1;
        code <<= 1;
    }
    return -1;
}

// RFC 1951 §3.2.5: lengths 3..258 (codes 257..285, index i = code - 257) and
// distances 1..32768 (codes 0..29).  Past the first few codes each group of
// four (lengths) or two (distances) codes doubles the step and adds an extra
// bit, so the table reduces to closed forms.
FAME_HD inline uint32_t infl_len_extra(uint32_t i) { return i < 8 || i == 28 ? 0u : (i - 4) >> 2; }
FAME_HD inline uint32_t infl_len_base(uint32_t i)
{
    if (i < 8) return 3 + i;
    if (i == 28) return 258;
    return ((4 + ((i - 4) & 3)) << infl_len_extra(i)) + 3;
}
FAME_HD inline uint32_t infl_dist_extra(uint32_t i) { return i < 4 ? 0u : (i - 2) >> 1; }
FAME_HD inline uint32_t infl_dist_base(uint32_t i) { return i < 4 ? 1 + i : ((2 + (i & 1)) << infl_dist_extra(i)) + 1; }

// Symbols of one compressed block into out[*pos ..), until end-of-block.
FAME_HD inline int infl_codes(InflBits& b, const InflCode& lit, const InflCode& dist, uint8_t* out, uint32_t cap,
                              uint32_t* pos)
{
    uint32_t p = *pos;
    for (;;) {
        const int s = infl_decode(b, lit);
        if (s < 0) return INFL_ERR_CODE;
        if (s < 256) {
            if (p >= cap) return INFL_ERR_SIZE;
            out[p++] = (uint8_t)s;
            continue;
        }
        if (s == 256) break;
        const uint32_t li = (uint32_t)s - 257;
        if (li >= 29) return INFL_ERR_CODE;
        uint32_t e;
        if (!infl_bits(b, infl_len_extra(li), e)) return INFL_ERR_INPUT;
        const uint32_t length = infl_len_base(li) + e;
        const int ds = infl_decode(b, dist);
        if (ds < 0 || ds >= 30) return INFL_ERR_CODE;
        if (!infl_bits(b, infl_dist_extra((uint32_t)ds), e)) return INFL_ERR_INPUT;
        const uint32_t d = infl_dist_base((uint32_t)ds) + e;
        if (d > p) return INFL_ERR_DIST;
        if (length > cap - p) return INFL_ERR_SIZE;
        for (uint32_t i = 0; i < length; ++i, ++p) out[p] = out[p - d];   // overlapping copies repeat
    }
    *pos = p;
    return INFL_OK;
}

// One raw DEFLATE stream: in[0 .. in_len) into out[0 .. cap); *out_len the
// bytes written.  sc: the code tables (3.6 KB).
FAME_HD inline int infl_raw(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len,
                            InflScratch& sc)
{
    InflBits b{in, in_len, 0, 0, 0};
    InflCode& lit = sc.lit;
    InflCode& dist = sc.dist;
    uint8_t* lens = sc.lens;
    uint32_t p = 0;
    uint32_t last = 0;
    *out_len = 0;
    do {
        uint32_t type;
        if (!infl_bits(b, 1, last) || !infl_bits(b, 2, type)) return INFL_ERR_INPUT;
        if (type == 0) {
            // stored: skip to a byte boundary; LEN, NLEN, then LEN bytes
            const uint32_t drop = b.cnt & 7u;
            b.buf >>= drop;
            b.cnt -= drop;
            uint32_t len, nlen;
            if (!infl_bits(b, 16, len) || !infl_bits(b, 16, nlen)) return INFL_ERR_INPUT;
            if ((len ^ 0xffffu) != nlen) return INFL_ERR_BLOCK;
            if (len > cap - p) return INFL_ERR_SIZE;
            for (uint32_t i = 0; i < len; ++i) {
                uint32_t v;
                if (!infl_bits(b, 8, v)) return INFL_ERR_INPUT;
                out[p++] = (uint8_t)v;
            }
        } else if (type == 1) {
            for (uint32_t s = 0; s < 288; ++s) lens[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
            for (uint32_t s = 0; s < 30; ++s) lens[288 + s] = 5;
            if (!infl_build(lit, lens, 288) || !infl_build(dist, lens + 288, 30)) return INFL_ERR_CODE;
            const int r = infl_codes(b, lit, dist, out, cap, &p);
            if (r) return r;
        } else if (type == 2) {
            uint32_t hlit, hdist, hclen;
            if (!infl_bits(b, 5, hlit) || !infl_bits(b, 5, hdist) || !infl_bits(b, 4, hclen)) return INFL_ERR_INPUT;
            hlit += 257;
            hdist += 1;
            hclen += 4;
            if (hlit > 286 || hdist > 30) return INFL_ERR_CODE;
            // code lengths of the code-length code, in the format's order
            const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19];
            for (int i = 0; i < 19; ++i) cl[i] = 0;
            for (uint32_t i = 0; i < hclen; ++i) {
                uint32_t v;
                if (!infl_bits(b, 3, v)) return INFL_ERR_INPUT;
                cl[order[i]] = (uint8_t)v;
            }
            if (!infl_build(lit, cl, 19)) return INFL_ERR_CODE;   // lit holds the code-length code for now
            uint32_t n = 0;
            while (n < hlit + hdist) {
                const int s = infl_decode(b, lit);
                if (s < 0) return INFL_ERR_CODE;
                if (s < 16) {
                    lens[n++] = (uint8_t)s;
                    continue;
                }
                uint32_t rep, v = 0;
                if (s == 16) {
                    if (n == 0) return INFL_ERR_CODE;
                    v = lens[n - 1];
                    if (!infl_bits(b, 2, rep)) return INFL_ERR_INPUT;
                    rep += 3;
                } else if (s == 17) {
                    if (!infl_bits(b, 3, rep)) return INFL_ERR_INPUT;
                    rep += 3;
                } else {
                    if (!infl_bits(b, 7, rep)) return INFL_ERR_INPUT;
                    rep += 11;
                }
                if (n + rep > hlit + hdist) return INFL_ERR_CODE;
                while (rep--) lens[n++] = (uint8_t)v;
            }
            if (lens[256] == 0) return INFL_ERR_CODE;   // no end-of-block code
            if (!infl_build(lit, lens, hlit) || !infl_build(dist, lens + hlit, hdist)) return INFL_ERR_CODE;
            const int r = infl_codes(b, lit, dist, out, cap, &p);
            if (r) return r;
        } else {
            return INFL_ERR_BLOCK;
        }
    } while (!last);
    *out_len = p;
    return INFL_OK;
}

// CRC-32 (reflected, polynomial 0xEDB88320) of data, bit by bit per byte
// through a 256-entry table the caller builds with crc32_table.
FAME_HD inline void crc32_table(uint32_t* t)
{
    for (uint32_t i = 0; i < 256; ++i) {
        uint32_t c = i;
        for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        t[i] = c;
    }
}

FAME_HD inline uint32_t crc32_of(const uint32_t* t, const uint8_t* p, uint32_t n)
{
    uint32_t c = 0xffffffffu;
    for (uint32_t i = 0; i < n; ++i) c = t[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    return c ^ 0xffffffffu;
}

// A BGZF member at m[0 .. avail): its total size (BSIZE + 1), or 0 when the
// header is not BGZF's (gzip, deflate, FEXTRA with a 'BC' subfield of 2
// bytes), the trailer declares more than 64 KiB of output, or the member is
// not complete in avail.  Sets the raw stream's
// offset and length and the trailer's CRC-32 and ISIZE.
FAME_HD inline uint32_t bgzf_member(const uint8_t* m, uint64_t avail, uint32_t* cdata, uint32_t* clen, uint32_t* crc,
                                    uint32_t* isize)
{
    if (avail < 18 || m[0] != 31 || m[1] != 139 || m[2] != 8 || !(m[3] & 4)) return 0;
    const uint32_t xlen = m[10] | (uint32_t)m[11] << 8;
    if (12ull + xlen > avail) return 0;
    uint32_t bsize = 0;
    bool found = false;
    for (uint32_t x = 12; x + 4 <= 12 + xlen;) {
        const uint32_t slen = m[x + 2] | (uint32_t)m[x + 3] << 8;
        if (m[x] == 'B' && m[x + 1] == 'C' && slen == 2 && x + 6 <= 12 + xlen) {
            bsize = m[x + 4] | (uint32_t)m[x + 5] << 8;
            found = true;
        }
        x += 4 + slen;
    }
    if (!found) return 0;
    const uint32_t total = bsize + 1;
    // the header (FEXTRA only: other optional fields are not part of the BGZF layout) and the 8-byte trailer
    if (total < 12 + xlen + 8 || total > avail || (m[3] & ~4u)) return 0;
    const uint8_t* tr = m + total - 8;
    *cdata = 12 + xlen;
    *clen = total - 8 - (12 + xlen);
    *crc = tr[0] | (uint32_t)tr[1] << 8 | (uint32_t)tr[2] << 16 | (uint32_t)tr[3] << 24;
    *isize = tr[4] | (uint32_t)tr[5] << 8 | (uint32_t)tr[6] << 16 | (uint32_t)tr[7] << 24;
    if (*isize > 65536) return 0;   // a BGZF member holds at most 64 KiB
    return total;
}

}  // namespace fame
