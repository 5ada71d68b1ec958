// Index build on the GPU: the tables of fame_index_build -- the reference's
// RefGenome constructor: window hashing and the bucket fill
// (RefGenome.cpp:532-759), filterHashTable (RefGenome.cpp:2267-2352),
// filterRedundancyInHashTable (RefGenome.cpp:2191-2264) and the T masks that
// save() writes (RefGenome.h:62-100) -- identical byte for byte, with every
// pass over the k-mers on the device:
//
//   1. one block per window: its N-free intervals and the spaced-seed hash of
//      every k-mer, numbered in the reference's insertion order (interval,
//      reverse strand before forward, position).  The first pass counts
//      bucket sizes, the second writes one 64-bit entry per k-mer {window,
//      insertion index, offset, strand} through per-bucket atomic cursors;
//   2. per bucket, the entries in reverse insertion order (descending entry
//      value) and the two filters: one thread per bucket up to IB_SMALL
//      entries, one block per bucket in shared memory below KMERCUTOFF, one
//      block per bucket with global scratch above;
//   3. compaction by a scan over the surviving entries, strandTable and the
//      T masks.
//
// The host keeps readReference and generateWindows (linear and cheap) and
// takes the finished tables back into a fame_host_index.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fame_gpu.h"
#include "dev_common.cuh"
#include "fame_const.h"
#include "index_host.h"

using namespace fame;

namespace {

constexpr unsigned FULL_MASK = 0xffffffffu;
constexpr uint32_t IB_SMALL = 16;        // bucket entries handled by one thread
constexpr uint32_t IB_MID_CAP = 2048;    // bucket entries handled by one block in shared memory
constexpr uint32_t IB_MAX_LONG = 64;     // N-free intervals of at least READLEN bases in a window (at most 60)
constexpr int SCAN_T = 256, SCAN_I = 16;
constexpr uint64_t SCAN_TILE = (uint64_t)SCAN_T * SCAN_I;

struct IbGenome {
    const uint8_t* seq;       // normalised chromosomes (ACGTN) back to back
    const uint64_t* off;      // start of each chromosome in seq
    const uint64_t* len;
    const uint64_t* t_msb;    // per chromosome, 'T' bits, most significant bit first in each word
    const uint64_t* a_lsb;    // 'A' bits, least significant bit first
    const uint64_t* poff;     // first word of each chromosome's bit planes
    const uint2* win;         // {start_pos, chrom} per window
    uint64_t n_win;
    uint32_t readlen;
};

// Fields of a bucket entry: window (63-32), insertion index in the window
// (31-16), offset in the window (15-1), forward strand (0).
__device__ __forceinline__ uint32_t e_win(uint64_t e) { return (uint32_t)(e >> 32); }
__device__ __forceinline__ uint32_t e_off(uint64_t e) { return (uint32_t)(e >> 1) & 0x7fffu; }
__device__ __forceinline__ uint32_t e_fwd(uint64_t e) { return (uint32_t)e & 1u; }
__device__ __forceinline__ bool same_run(uint64_t a, uint64_t b) { return e_win(a) == e_win(b) && e_fwd(a) == e_fwd(b); }

// bit 31 - i: 'T' at s + i (i < 32); positions past the chromosome are 0
__device__ __forceinline__ uint32_t ib_t_fwd(const IbGenome& G, uint32_t c, uint64_t s)
{
    const uint64_t* b = G.t_msb + G.poff[c];
    const uint64_t w = s >> 6, r = s & 63;
    const uint64_t x = r ? (b[w] << r) | (b[w + 1] >> (64 - r)) : b[w];
    return (uint32_t)(x >> 32);
}

// bit j: 'A' at s + j (j < 32)
__device__ __forceinline__ uint32_t ib_a_lo(const IbGenome& G, uint32_t c, uint64_t s)
{
    const uint64_t* b = G.a_lsb + G.poff[c];
    const uint64_t w = s >> 6, r = s & 63;
    const uint64_t x = r ? (b[w] >> r) | (b[w + 1] << (64 - r)) : b[w];
    return (uint32_t)x;
}

// reproduceTMask (RefGenome.cpp:2135-2189)
__device__ __forceinline__ uint32_t ib_tmask(const IbGenome& G, uint64_t e)
{
    const uint2 w = G.win[e_win(e)];
    const uint64_t s0 = (uint64_t)w.x + e_off(e);
    return e_fwd(e) ? ib_t_fwd(G, w.y, s0) : ib_a_lo(G, w.y, s0);
}

// reproduceKmerSeq (RefGenome.cpp:2028-2132): 2 bits per seeded position
__device__ uint64_t ib_kmer_seq(const IbGenome& G, uint64_t e)
{
    const uint2 w = G.win[e_win(e)];
    const uint64_t s0 = (uint64_t)w.x + e_off(e), L = G.len[w.y];
    const uint8_t* g = G.seq + G.off[w.y];
    const bool fwd = e_fwd(e);
    uint64_t k = 0;
#pragma unroll 4
    for (uint32_t i = 0; i < KMERLEN; ++i) {
        k <<= 2;
        if (!((SEEDBITS >> (31 - i)) & 1u)) continue;
        const uint64_t p = fwd ? s0 + i : s0 + KMERLEN - 1 - i;
        const uint8_t ch = p < L ? g[p] : 'N';
        if (fwd) k += (ch == 'C' || ch == 'T') ? 3 : ch == 'G' ? 2 : 0;
        else k += (ch == 'G' || ch == 'A') ? 3 : ch == 'C' ? 2 : 0;
    }
    return k;
}

// ---- block-wide helpers ----------------------------------------------------
template <int NT>
__device__ uint64_t block_excl_sum(uint64_t v, uint64_t* total)
{
    __shared__ uint64_t ws[NT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint64_t t = __shfl_up_sync(FULL_MASK, inc, d);
        if (lane >= d) inc += t;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint64_t x = lane < NT / 32 ? ws[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t t = __shfl_up_sync(FULL_MASK, x, d);
            if (lane >= d) x += t;
        }
        if (lane < NT / 32) ws[lane] = x;
    }
    __syncthreads();
    const uint64_t pre = (warp ? ws[warp - 1] : 0) + inc - v;
    if (total) *total = ws[NT / 32 - 1];
    __syncthreads();
    return pre;
}

template <int NT>
__device__ int block_incl_max(int v, int* block_max)
{
    __shared__ int wm[NT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(FULL_MASK, inc, d);
        if (lane >= d) inc = max(inc, t);
    }
    if (lane == 31) wm[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int x = lane < NT / 32 ? wm[lane] : -1;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(FULL_MASK, x, d);
            if (lane >= d) x = max(x, t);
        }
        if (lane < NT / 32) wm[lane] = x;
    }
    __syncthreads();
    const int r = warp ? max(wm[warp - 1], inc) : inc;
    *block_max = wm[NT / 32 - 1];
    __syncthreads();
    return r;
}

// Bitonic sort of P (a power of two) values by the whole block; descending
// or ascending.  The caller synchronises before (the values are in place).
template <bool DESC, class T>
__device__ void block_bitonic(T* v, uint32_t P)
{
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const T a = v[i], b = v[l];
                    const bool up = ((i & k) == 0) != DESC;   // this pair's direction: ascending?
                    if (up ? a > b : a < b) { v[i] = b; v[l] = a; }
                }
            }
            __syncthreads();
        }
    }
}

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

__device__ __forceinline__ uint32_t pow2_at_least(uint32_t n)
{
    uint32_t p = 1;
    while (p < n) p <<= 1;
    return p;
}

// ---- 1. genome bit planes and window k-mers ---------------------------------
// 'T' and 'A' bit planes of chromosome c (words past the end stay 0).
__global__ void k_ib_planes(const uint8_t* seq, uint64_t len, uint64_t words, uint64_t* t_msb, uint64_t* a_lsb)
{
    for (uint64_t wd = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; wd < words; wd += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t t = 0, a = 0;
        const uint64_t p0 = wd * 64;
        for (uint32_t i = 0; i < 64 && p0 + i < len; ++i) {
            const uint8_t ch = seq[p0 + i];
            if (ch == 'T') t |= 1ull << (63 - i);
            else if (ch == 'A') a |= 1ull << i;
        }
        t_msb[wd] = t;
        a_lsb[wd] = a;
    }
}

// Every k-mer of every window, in the reference's insertion order
// (RefGenome.cpp:621-759).  FILL = false: count per bucket into cur;
// FILL = true: write the entries at the buckets' cursors.
template <bool FILL>
__global__ void __launch_bounds__(256) k_ib_window_kmers(IbGenome G, uint32_t* cur, uint64_t* ent)
{
    __shared__ uint8_t raw[WINLEN], red[WINLEN], redr[WINLEN];
    __shared__ uint16_t ivs[WINLEN / 2 + 1], ive[WINLEN / 2 + 1];
    __shared__ uint16_t lfirst[IB_MAX_LONG], lsecond[IB_MAX_LONG];
    __shared__ uint32_t lbase[IB_MAX_LONG + 1], lnq[IB_MAX_LONG];
    __shared__ uint32_t s_nl;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (uint64_t w = blockIdx.x; w < G.n_win; w += gridDim.x) {
        const uint2 wi = G.win[w];
        const uint64_t sp = wi.x, L = G.len[wi.y];
        const uint32_t n = (uint32_t)umin64(WINLEN, L - sp);   // windows start inside their chromosome
        const uint8_t* g = G.seq + G.off[wi.y] + sp;
        for (uint32_t j = tid; j < WINLEN; j += blockDim.x) raw[j] = j < n ? g[j] : 0;
        __syncthreads();
        for (uint32_t j = tid; j < WINLEN; j += blockDim.x) {
            // forward buffer (C read as T): the base at j, unless an N at the
            // mirrored position WINLEN - 1 - j came later in the reference's
            // loop, which stores that N into the forward buffer
            const uint32_t m = WINLEN - 1 - j;
            const bool mirror_n = m < n && raw[m] == 'N';
            uint8_t f = 0;
            if (j < n && !(mirror_n && m > j)) f = raw[j] == 'C' ? (uint8_t)'T' : raw[j];
            else if (mirror_n) f = 'N';
            red[j] = f;
            // reverse buffer: complement of the base at j, stored at WINLEN - 1 - j (N leaves 0)
            const uint8_t ch = j < n ? raw[j] : 0;
            redr[m] = ch == 'C' ? 'G' : ch == 'G' ? 'T' : ch == 'T' ? 'A' : ch == 'A' ? 'T' : 0;
        }
        __syncthreads();
        if (warp == 0) {
            // N-free intervals [ivs, ive] in order
            uint32_t ns = 0, ne = 0;
            const unsigned lt = (1u << lane) - 1;
            for (uint32_t b = 0; b < n; b += 32) {
                const uint32_t j = b + lane;
                const bool ok = j < n && raw[j] != 'N';
                const bool okp = j > 0 && j - 1 < n && raw[j - 1] != 'N';
                const bool okn = j + 1 < n && raw[j + 1] != 'N';
                const bool st = ok && !okp, en = ok && !okn;
                const unsigned bs = __ballot_sync(FULL_MASK, st), be = __ballot_sync(FULL_MASK, en);
                if (st) ivs[ns + __popc(bs & lt)] = (uint16_t)j;
                if (en) ive[ne + __popc(be & lt)] = (uint16_t)j;
                ns += __popc(bs);
                ne += __popc(be);
            }
            __syncwarp();
            // intervals of at least READLEN bases: k-mers per strand and the
            // insertion index of their first k-mer
            uint32_t nl = 0, base = 0;
            for (uint32_t q0 = 0; q0 < ns; q0 += 32) {
                const uint32_t q = q0 + lane;
                const uint32_t d = q < ns ? (uint32_t)ive[q] - ivs[q] + 1 : 0;
                const bool lg = q < ns && d >= G.readlen;
                const unsigned bl = __ballot_sync(FULL_MASK, lg);
                // the first k-mer, then one every SKIPMOD rolls (RefGenome.cpp:736-755)
                const uint32_t nq = lg ? 1 + (d - KMERLEN + SKIPMOD - 1) / SKIPMOD : 0;
                uint32_t inc = 2 * nq;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(FULL_MASK, inc, o);
                    if (lane >= (uint32_t)o) inc += t;
                }
                const uint32_t r = nl + __popc(bl & lt);
                if (lg && r < IB_MAX_LONG) {
                    lfirst[r] = ivs[q];
                    lsecond[r] = ive[q];
                    lnq[r] = nq;
                    lbase[r] = base + inc - 2 * nq;
                }
                nl += __popc(bl);
                base += __shfl_sync(FULL_MASK, inc, 31);
            }
            if (lane == 0) {
                s_nl = min(nl, IB_MAX_LONG);
                lbase[min(nl, IB_MAX_LONG)] = base;
            }
        }
        __syncthreads();
        const uint32_t nl = s_nl, total = lbase[nl];
        for (uint32_t e = tid; e < total; e += blockDim.x) {
            uint32_t q = 0;
            while (q + 1 < nl && lbase[q + 1] <= e) ++q;
            const uint32_t ue = e - lbase[q], nq = lnq[q];
            const uint32_t fwd = ue < nq ? 0u : 1u;   // the reverse strand first
            const uint32_t u = ue - fwd * nq;
            const uint32_t t = u == 0 ? 0u : (u - 1) * SKIPMOD + 1;
            const uint32_t first = lfirst[q], second = lsecond[q];
            const uint8_t* s = fwd ? red + first + t : redr + (WINLEN - 1 - second) + t;
            uint64_t h = 0;
#pragma unroll
            for (uint32_t x = 0; x < KMERLEN; ++x)
                if ((SEEDBITS >> (31 - x)) & 1u) h ^= rotl64(nt_val(s[x]), 31 - x);
            const uint32_t key = (uint32_t)h & HTAB_MASK;
            const uint32_t kp = fwd ? first + t : WINLEN - first - KMERLEN - t;
            const uint32_t slot = atomicAdd(cur + key, 1u);
            if (FILL) ent[slot] = (w << 32) | ((uint64_t)e << 16) | ((uint64_t)kp << 1) | fwd;
        }
        __syncthreads();
    }
}

// ---- scans --------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(SCAN_T) k_ib_tile_sums(const T* in, uint64_t n, uint64_t* tsum)
{
    const uint64_t t0 = blockIdx.x * SCAN_TILE, t1 = umin64(n, t0 + SCAN_TILE);
    uint64_t s = 0;
    for (uint64_t i = t0 + threadIdx.x; i < t1; i += SCAN_T) s += in[i];
    uint64_t tot;
    block_excl_sum<SCAN_T>(s, &tot);
    if (threadIdx.x == 0) tsum[blockIdx.x] = tot;
}

// exclusive scan of nt tile sums in place; the total at tsum[nt]
__global__ void __launch_bounds__(1024) k_ib_scan_sums(uint64_t* tsum, uint64_t nt)
{
    const uint64_t per = (nt + 1023) / 1024, b = umin64(nt, threadIdx.x * per), e = umin64(nt, b + per);
    uint64_t s = 0;
    for (uint64_t i = b; i < e; ++i) s += tsum[i];
    uint64_t tot;
    uint64_t run = block_excl_sum<1024>(s, &tot);
    for (uint64_t i = b; i < e; ++i) {
        const uint64_t v = tsum[i];
        tsum[i] = run;
        run += v;
    }
    if (threadIdx.x == 0) tsum[nt] = tot;
}

// out[i] = sum of in[0 .. i) (uint32; the caller checks the total fits)
template <class T>
__global__ void __launch_bounds__(SCAN_T) k_ib_scan_apply(const T* in, uint64_t n, const uint64_t* tsum, uint32_t* out)
{
    const uint64_t i0 = blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_I;
    uint64_t s = 0;
    for (uint64_t i = i0; i < umin64(n, i0 + SCAN_I); ++i) s += in[i];
    uint64_t run = tsum[blockIdx.x] + block_excl_sum<SCAN_T>(s, nullptr);
    for (uint64_t i = i0; i < umin64(n, i0 + SCAN_I); ++i) {
        const uint64_t v = in[i];
        out[i] = (uint32_t)run;
        run += v;
    }
}

// ---- 2. bucket order and filters ------------------------------------------------
// One thread per bucket of up to IB_SMALL entries; larger buckets go to the
// block passes' lists.
__global__ void __launch_bounds__(256) k_ib_bucket_small(IbGenome G, const uint32_t* tab, uint64_t* ent, uint8_t* keep,
                                                         uint32_t* kept, uint32_t* mid, uint32_t* n_mid, uint32_t* big,
                                                         uint32_t* n_big, int noloss)
{
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < HTABSIZE; b += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s0 = tab[b], n = tab[b + 1] - s0;
        if (n > IB_SMALL) {
            kept[b] = 0;   // the block passes write it
            if (n <= IB_MID_CAP && (noloss || n < KMERCUTOFF)) mid[atomicAdd(n_mid, 1u)] = (uint32_t)b;
            else big[atomicAdd(n_big, 1u)] = (uint32_t)b;
            continue;
        }
        if (n <= 1) {
            kept[b] = n;
            if (n) keep[s0] = 1;
            continue;
        }
        uint64_t e[IB_SMALL];
        uint32_t tm[IB_SMALL];
        for (uint32_t i = 0; i < n; ++i) {
            // insertion sort, descending: reverse insertion order
            const uint64_t v = ent[s0 + i];
            uint32_t j = i;
            while (j > 0 && e[j - 1] < v) { e[j] = e[j - 1]; --j; }
            e[j] = v;
        }
        uint32_t k = 0;
        for (uint32_t i = 0; i < n; ++i) {
            ent[s0 + i] = e[i];
            tm[i] = ib_tmask(G, e[i]);
            // filterRedundancyInHashTable: dropped when an earlier entry of the
            // same window and strand run has the same T mask
            bool kp = true;
            for (int j = (int)i - 1; j >= 0; --j) {
                if (!same_run(e[j], e[i])) break;
                if (tm[j] == tm[i]) { kp = false; break; }
            }
            keep[s0 + i] = kp;
            k += kp;
        }
        kept[b] = k;
    }
}

// One block per bucket of up to IB_MID_CAP entries and below KMERCUTOFF
// (or any size up to IB_MID_CAP without the k-mer filter), in shared memory.
__global__ void __launch_bounds__(128) k_ib_bucket_mid(IbGenome G, const uint32_t* tab, uint64_t* ent, uint8_t* keep,
                                                       uint32_t* kept, const uint32_t* mid, const uint32_t* n_mid)
{
    __shared__ uint64_t sh[IB_MID_CAP];
    __shared__ uint32_t tms[IB_MID_CAP];
    __shared__ uint32_t s_cnt;
    const uint32_t nm = *n_mid;
    for (uint32_t x = blockIdx.x; x < nm; x += gridDim.x) {
        const uint32_t b = mid[x], s0 = tab[b], n = tab[b + 1] - s0;
        const uint32_t P = pow2_at_least(n);   // n <= IB_MID_CAP
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) sh[i] = i < n ? ent[s0 + i] : 0ull;
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        block_bitonic<true>(sh, P);
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            ent[s0 + i] = sh[i];
            tms[i] = ib_tmask(G, sh[i]);
        }
        __syncthreads();
        uint32_t k = 0;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            bool kp = true;
            for (int j = (int)i - 1; j >= 0; --j) {
                if (!same_run(sh[j], sh[i])) break;
                if (tms[j] == tms[i]) { kp = false; break; }
            }
            keep[s0 + i] = kp;
            k += kp;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) k += __shfl_xor_sync(FULL_MASK, k, d);
        if ((threadIdx.x & 31) == 0) atomicAdd(&s_cnt, k);
        __syncthreads();
        if (threadIdx.x == 0) kept[b] = s_cnt;
        __syncthreads();
    }
}

// One block per large bucket with scratch in global memory (32 bytes per
// entry, rounded up to a power of two, at boff[x] in 8-byte words): the
// KMERCUTOFF filter (filterHashTable) as well, recording each filtered k-mer
// once, at its first occurrence in bucket order, as {bucket << 32 | rank, k-mer}.
__global__ void __launch_bounds__(256) k_ib_bucket_big(IbGenome G, const uint32_t* tab, uint64_t* ent, uint8_t* keep,
                                                       uint32_t* kept, const uint32_t* blist, const uint64_t* boff,
                                                       uint32_t nb, uint64_t* scratch, int noloss, ulonglong2* filt,
                                                       unsigned long long* n_filt, uint64_t filt_cap)
{
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_cnt;
    for (uint32_t x = blockIdx.x; x < nb; x += gridDim.x) {
        const uint32_t b = blist[x], s0 = tab[b], n = tab[b + 1] - s0;
        const uint32_t P = pow2_at_least(n);
        uint64_t* A = scratch + boff[x];                 // entries, sorted
        uint64_t* K = A + P;                             // k-mer sequences, sorted
        uint32_t* tm = (uint32_t*)(A + 2ull * P);        // T masks
        uint32_t* mn = tm + P;                           // first occurrence of each filtered sequence
        int* pk = (int*)(mn + P);                        // last entry kept by the k-mer filter, up to i
        uint8_t* k1 = (uint8_t*)(pk + P);                // kept by the k-mer filter
        for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) A[i] = i < n ? ent[s0 + i] : 0ull;
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        block_bitonic<true>(A, P);
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            ent[s0 + i] = A[i];
            tm[i] = ib_tmask(G, A[i]);
            k1[i] = 1;
        }
        __syncthreads();
        if (!noloss && n >= KMERCUTOFF) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                K[i] = i < n ? ib_kmer_seq(G, A[i]) : ~0ull;   // no k-mer sequence has all 64 bits set
                mn[i] = 0xffffffffu;
            }
            __syncthreads();
            block_bitonic<false>(K, P);
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                const uint64_t ks = ib_kmer_seq(G, A[i]);
                uint32_t lo = 0, hi = n;
                while (lo < hi) { const uint32_t m = (lo + hi) >> 1; if (K[m] < ks) lo = m + 1; else hi = m; }
                const uint32_t lb = lo;
                hi = n;
                while (lo < hi) { const uint32_t m = (lo + hi) >> 1; if (K[m] <= ks) lo = m + 1; else hi = m; }
                if (lo - lb >= KMERCUTOFF) {
                    k1[i] = 0;
                    atomicMin(&mn[lb], i);
                }
            }
            __syncthreads();
            // the filtered sequences in order of first occurrence
            uint64_t rank0 = 0;
            for (uint32_t c0 = 0; c0 < n; c0 += blockDim.x) {
                const uint32_t i = c0 + threadIdx.x;
                uint64_t ks = 0;
                bool first = false;
                if (i < n && !k1[i]) {
                    ks = ib_kmer_seq(G, A[i]);
                    uint32_t lo = 0, hi = n;
                    while (lo < hi) { const uint32_t m = (lo + hi) >> 1; if (K[m] < ks) lo = m + 1; else hi = m; }
                    first = mn[lo] == i;
                }
                uint64_t tot;
                const uint64_t r = block_excl_sum<256>(first ? 1 : 0, &tot);
                if (threadIdx.x == 0 && tot) s_base = atomicAdd(n_filt, (unsigned long long)tot);
                __syncthreads();
                if (first && s_base + r < filt_cap)
                    filt[s_base + r] = make_ulonglong2(((unsigned long long)b << 32) | (rank0 + r), ks);
                rank0 += tot;
                __syncthreads();
            }
        }
        // pk[i]: the last index <= i kept by the k-mer filter (-1: none)
        int carry = -1;
        for (uint32_t c0 = 0; c0 < n; c0 += blockDim.x) {
            const uint32_t i = c0 + threadIdx.x;
            int bm;
            const int v = block_incl_max<256>(i < n && k1[i] ? (int)i : -1, &bm);
            if (i < n) pk[i] = max(v, carry);
            carry = max(carry, bm);
        }
        __syncthreads();
        // filterRedundancyInHashTable over the entries the k-mer filter kept
        uint32_t k = 0;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            bool kp = k1[i];
            if (kp) {
                for (int j = i > 0 ? pk[i - 1] : -1; j >= 0; j = j > 0 ? pk[j - 1] : -1) {
                    if (!same_run(A[j], A[i])) break;
                    if (tm[j] == tm[i]) { kp = false; break; }
                }
            }
            keep[s0 + i] = kp;
            k += kp;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) k += __shfl_xor_sync(FULL_MASK, k, d);
        if ((threadIdx.x & 31) == 0) atomicAdd(&s_cnt, k);
        __syncthreads();
        if (threadIdx.x == 0) kept[b] = s_cnt;
        __syncthreads();
    }
}

// sizes of the listed buckets
__global__ void k_ib_list_sizes(const uint32_t* tab, const uint32_t* list, uint32_t n, uint32_t* sizes)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x)
        sizes[x] = tab[list[x] + 1] - tab[list[x]];
}

// ---- 3. compaction, strandTable, T masks --------------------------------------------
__global__ void __launch_bounds__(SCAN_T) k_ib_compact(const uint64_t* ent, const uint8_t* keep, uint64_t n,
                                                      const uint64_t* tsum, uint32_t* kmeta, uint8_t* kstr, uint16_t* koff)
{
    const uint64_t i0 = blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_I, i1 = umin64(n, i0 + SCAN_I);
    uint64_t s = 0;
    for (uint64_t i = i0; i < i1; ++i) s += keep[i];
    uint64_t o = tsum[blockIdx.x] + block_excl_sum<SCAN_T>(s, nullptr);
    for (uint64_t i = i0; i < i1; ++i) {
        if (!keep[i]) continue;
        const uint64_t e = ent[i];
        kmeta[o] = e_win(e);
        kstr[o] = (uint8_t)e_fwd(e);
        koff[o] = (uint16_t)e_off(e);
        ++o;
    }
}

__global__ void k_ib_strand_bits(const uint8_t* kstr, uint64_t nk, uint8_t* bits)
{
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < (nk + 7) / 8; j += (uint64_t)gridDim.x * blockDim.x) {
        uint8_t v = 0;
        for (uint64_t i = 8 * j; i < umin64(8 * j + 8, nk); ++i)
            if (kstr[i]) v |= (uint8_t)(1u << (i & 7));
        bits[j] = v;
    }
}

// getTMask at save time (RefGenome.h:62-100): the strand is read at
// strandTable[window id]; the reverse loop skips base 0.
__global__ void k_ib_tmask_save(IbGenome G, const uint32_t* kmeta, const uint8_t* kstr, const uint16_t* koff, uint64_t nk,
                                uint2* kmer)
{
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nk; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t w = kmeta[k];
        const uint2 wi = G.win[w];
        const uint64_t s0 = (uint64_t)wi.x + koff[k];
        const bool fwd = w < nk ? kstr[w] != 0 : false;
        kmer[k] = make_uint2(w, fwd ? ib_t_fwd(G, wi.y, s0) : (ib_a_lo(G, wi.y, s0 + 1) & 0x7fffffffu));
    }
}

// ---- host ----------------------------------------------------------------------------
struct DevBufs {
    std::vector<void*> p;
    ~DevBufs() { for (void* x : p) cudaFree(x); }
    template <class T> bool alloc(T** out, uint64_t count)
    {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<uint64_t>(16, count * sizeof(T))) != cudaSuccess) return false;
        p.push_back(q);
        *out = (T*)q;
        return true;
    }
    void release(void* q)
    {
        for (auto& x : p)
            if (x == q) { cudaFree(x); x = nullptr; }
    }
};

struct IbFail {
    int code;
};

}  // namespace

extern "C" int fame_index_build_gpu(uint32_t readlen, uint32_t n_chrom, const char* const* seq, const uint64_t* len,
                                    const char* const* names, int noloss, int device, fame_host_index** out)
{
    if (!out || !seq || !len || n_chrom == 0 || n_chrom > 256 || readlen <= KMERLEN || readlen >= WINLEN) return FAME_ERR_ARG;
    *out = nullptr;
    const bool timing = std::getenv("FAME_INDEX_TIMING") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* name) {
        if (!timing) return;
        cudaDeviceSynchronize();
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "fame_index_build_gpu: %-22s %8.2f s\n", name, std::chrono::duration<double>(now - t_last).count());
        t_last = now;
    };
    fame_host_index* ix = new (std::nothrow) fame_host_index();
    if (!ix) return FAME_ERR_NOMEM;
    int prev_dev = 0;
    cudaGetDevice(&prev_dev);
    try {
        auto ck = [](cudaError_t e, int code = FAME_ERR_CUDA) { if (e != cudaSuccess) throw IbFail{code}; };
        auto launched = [&]() { ck(cudaGetLastError()); };
        ck(cudaSetDevice(device));
        int sms = 1;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        index_build_front(ix, readlen, n_chrom, seq, len, names, (int)std::max(1u, std::thread::hardware_concurrency()));
        phase("sequences, CpGs, windows");
        DevBufs B;
        auto need = [&](bool ok) { if (!ok) throw IbFail{FAME_ERR_NOMEM}; };
        // genome, offsets, bit planes, windows
        std::vector<uint64_t> off(n_chrom), clen(n_chrom), poff(n_chrom + 1, 0);
        uint64_t tot = 0;
        for (uint32_t c = 0; c < n_chrom; ++c) {
            off[c] = tot;
            clen[c] = ix->seq[c].size();
            tot += clen[c];
            poff[c + 1] = poff[c] + (clen[c] + 2 * WINLEN) / 64 + 2;
        }
        uint8_t* d_seq; uint64_t *d_off, *d_len, *d_poff, *d_t, *d_a; uint2* d_win;
        need(B.alloc(&d_seq, tot) && B.alloc(&d_off, n_chrom) && B.alloc(&d_len, n_chrom) && B.alloc(&d_poff, n_chrom + 1) &&
             B.alloc(&d_t, poff[n_chrom]) && B.alloc(&d_a, poff[n_chrom]) && B.alloc(&d_win, ix->win.size()));
        for (uint32_t c = 0; c < n_chrom; ++c)
            if (clen[c]) ck(cudaMemcpy(d_seq + off[c], ix->seq[c].data(), clen[c], cudaMemcpyHostToDevice));
        ck(cudaMemcpy(d_off, off.data(), 8ull * n_chrom, cudaMemcpyHostToDevice));
        ck(cudaMemcpy(d_len, clen.data(), 8ull * n_chrom, cudaMemcpyHostToDevice));
        ck(cudaMemcpy(d_poff, poff.data(), 8ull * (n_chrom + 1), cudaMemcpyHostToDevice));
        {
            std::vector<uint2> w(ix->win.size());
            for (size_t i = 0; i < w.size(); ++i) w[i] = make_uint2(ix->win[i].start_pos, ix->win[i].chrom);
            ck(cudaMemcpy(d_win, w.data(), 8ull * w.size(), cudaMemcpyHostToDevice));
        }
        for (uint32_t c = 0; c < n_chrom; ++c) {
            const uint64_t words = poff[c + 1] - poff[c];
            k_ib_planes<<<(unsigned)std::min<uint64_t>((words + 255) / 256, 8ull * sms), 256>>>(d_seq + off[c], clen[c], words,
                                                                                               d_t + poff[c], d_a + poff[c]);
            launched();
        }
        IbGenome G{d_seq, d_off, d_len, d_t, d_a, d_poff, d_win, ix->win.size(), readlen};
        phase("genome upload");
        // pass 1: bucket sizes; bucket starts
        const uint64_t NT_TAB = HTABSIZE / SCAN_TILE;
        uint32_t *d_cur, *d_tab;
        uint64_t* d_tsum;
        need(B.alloc(&d_cur, HTABSIZE + 1) && B.alloc(&d_tab, HTABSIZE + 1) && B.alloc(&d_tsum, NT_TAB + 1));
        ck(cudaMemset(d_cur, 0, 4 * (HTABSIZE + 1)));
        const unsigned wgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ix->win.size(), 8ull * sms));
        if (!ix->win.empty()) {
            k_ib_window_kmers<false><<<wgrid, 256>>>(G, d_cur, nullptr);
            launched();
        }
        phase("pass 1 (count)");
        k_ib_tile_sums<uint32_t><<<(unsigned)NT_TAB, SCAN_T>>>(d_cur, HTABSIZE, d_tsum);
        k_ib_scan_sums<<<1, 1024>>>(d_tsum, NT_TAB);
        k_ib_scan_apply<uint32_t><<<(unsigned)NT_TAB, SCAN_T>>>(d_cur, HTABSIZE, d_tsum, d_tab);
        launched();
        uint64_t total = 0;
        ck(cudaMemcpy(&total, d_tsum + NT_TAB, 8, cudaMemcpyDeviceToHost));
        if (total >= 0xffffffffull) throw IbFail{FAME_ERR_INDEX};
        {
            const uint32_t t32 = (uint32_t)total;
            ck(cudaMemcpy(d_tab + HTABSIZE, &t32, 4, cudaMemcpyHostToDevice));
        }
        ck(cudaMemcpy(d_cur, d_tab, 4 * (HTABSIZE + 1), cudaMemcpyDeviceToDevice));
        phase("bucket starts");
        // pass 2: entries
        uint64_t* d_ent;
        need(B.alloc(&d_ent, total));
        if (!ix->win.empty()) {
            k_ib_window_kmers<true><<<wgrid, 256>>>(G, d_cur, d_ent);
            launched();
        }
        phase("pass 2 (fill)");
        // bucket order and filters
        uint8_t* d_keep;
        uint32_t *d_kept = d_cur, *d_mid, *d_big, *d_nlist;   // cursors are done: kept counts take their place
        const uint64_t mid_cap = total / (IB_SMALL + 1) + 1, big_cap = total / KMERCUTOFF + 1;
        const uint64_t filt_cap = total / KMERCUTOFF + 1;
        ulonglong2* d_filt;
        unsigned long long* d_nfilt;
        need(B.alloc(&d_keep, total) && B.alloc(&d_mid, mid_cap) && B.alloc(&d_big, big_cap) && B.alloc(&d_nlist, 2) &&
             B.alloc(&d_filt, filt_cap) && B.alloc(&d_nfilt, 1));
        ck(cudaMemset(d_nlist, 0, 8));
        ck(cudaMemset(d_nfilt, 0, 8));
        k_ib_bucket_small<<<16u * sms, 256>>>(G, d_tab, d_ent, d_keep, d_kept, d_mid, d_nlist, d_big, d_nlist + 1, noloss);
        launched();
        k_ib_bucket_mid<<<16u * sms, 128>>>(G, d_tab, d_ent, d_keep, d_kept, d_mid, d_nlist);
        launched();
        uint32_t nlist[2];
        ck(cudaMemcpy(nlist, d_nlist, 8, cudaMemcpyDeviceToHost));
        if (nlist[1]) {
            // large buckets: scratch of 32 bytes per entry (power of two), in batches
            uint32_t* d_sz;
            need(B.alloc(&d_sz, nlist[1]));
            k_ib_list_sizes<<<(nlist[1] + 255) / 256, 256>>>(d_tab, d_big, nlist[1], d_sz);
            launched();
            std::vector<uint32_t> sz(nlist[1]), ids(nlist[1]);
            ck(cudaMemcpy(sz.data(), d_sz, 4ull * nlist[1], cudaMemcpyDeviceToHost));
            ck(cudaMemcpy(ids.data(), d_big, 4ull * nlist[1], cudaMemcpyDeviceToHost));
            std::vector<uint64_t> words(nlist[1]);
            uint64_t max_words = 0;
            for (uint32_t i = 0; i < nlist[1]; ++i) {
                uint64_t p = 1;
                while (p < sz[i]) p <<= 1;
                words[i] = 4 * p;
                max_words = std::max(max_words, words[i]);
            }
            const uint64_t cap_words = std::max<uint64_t>(max_words, 1ull << 28);   // 2 GiB, or the largest bucket
            uint64_t* d_scr;
            uint64_t* d_boff;
            uint32_t* d_blist;
            need(B.alloc(&d_scr, cap_words) && B.alloc(&d_boff, nlist[1]) && B.alloc(&d_blist, nlist[1]));
            for (uint32_t i0 = 0; i0 < nlist[1];) {
                std::vector<uint64_t> bo;
                std::vector<uint32_t> bl;
                uint64_t used = 0;
                uint32_t i1 = i0;
                while (i1 < nlist[1] && used + words[i1] <= cap_words) {
                    bo.push_back(used);
                    bl.push_back(ids[i1]);
                    used += words[i1];
                    ++i1;
                }
                ck(cudaMemcpy(d_boff, bo.data(), 8ull * bo.size(), cudaMemcpyHostToDevice));
                ck(cudaMemcpy(d_blist, bl.data(), 4ull * bl.size(), cudaMemcpyHostToDevice));
                k_ib_bucket_big<<<(unsigned)std::min<uint64_t>(bl.size(), 2ull * sms), 256>>>(
                    G, d_tab, d_ent, d_keep, d_kept, d_blist, d_boff, (uint32_t)bl.size(), d_scr, noloss, d_filt, d_nfilt,
                    filt_cap);
                launched();
                ck(cudaDeviceSynchronize());
                i0 = i1;
            }
        }
        phase("bucket order, filters");
        // compaction: new bucket starts from the kept counts, entries from a scan of the keep flags
        ck(cudaMemset(d_kept + HTABSIZE, 0, 4));
        k_ib_tile_sums<uint32_t><<<(unsigned)NT_TAB, SCAN_T>>>(d_kept, HTABSIZE, d_tsum);
        k_ib_scan_sums<<<1, 1024>>>(d_tsum, NT_TAB);
        launched();
        uint64_t nk = 0;
        ck(cudaMemcpy(&nk, d_tsum + NT_TAB, 8, cudaMemcpyDeviceToHost));
        k_ib_scan_apply<uint32_t><<<(unsigned)NT_TAB, SCAN_T>>>(d_kept, HTABSIZE, d_tsum, d_tab);   // the old starts are done
        launched();
        {
            const uint32_t n32 = (uint32_t)nk;
            ck(cudaMemcpy(d_tab + HTABSIZE, &n32, 4, cudaMemcpyHostToDevice));
        }
        const uint64_t NT_ENT = (total + SCAN_TILE - 1) / SCAN_TILE;
        uint64_t* d_etsum;
        uint32_t* d_kmeta;
        uint8_t* d_kstr;
        uint16_t* d_koff;
        need(B.alloc(&d_etsum, NT_ENT + 1) && B.alloc(&d_kmeta, nk) && B.alloc(&d_kstr, nk) && B.alloc(&d_koff, nk));
        if (total) {
            k_ib_tile_sums<uint8_t><<<(unsigned)NT_ENT, SCAN_T>>>(d_keep, total, d_etsum);
            k_ib_scan_sums<<<1, 1024>>>(d_etsum, NT_ENT);
            k_ib_compact<<<(unsigned)NT_ENT, SCAN_T>>>(d_ent, d_keep, total, d_etsum, d_kmeta, d_kstr, d_koff);
            launched();
            uint64_t nk2 = 0;
            ck(cudaMemcpy(&nk2, d_etsum + NT_ENT, 8, cudaMemcpyDeviceToHost));
            if (nk2 != nk) throw IbFail{FAME_ERR_INDEX};
        }
        B.release(d_ent);
        B.release(d_keep);
        phase("compaction");
        uint8_t* d_bits;
        uint2* d_kmer;
        need(B.alloc(&d_bits, (nk + 7) / 8) && B.alloc(&d_kmer, nk));
        if (nk) {
            k_ib_strand_bits<<<8u * sms, 256>>>(d_kstr, nk, d_bits);
            k_ib_tmask_save<<<16u * sms, 256>>>(G, d_kmeta, d_kstr, d_koff, nk, d_kmer);
            launched();
        }
        ck(cudaDeviceSynchronize());
        phase("strand bits, T masks");
        // tables back to the host
        ix->tab32.resize(HTABSIZE + 1);
        ck(cudaMemcpy(ix->tab32.data(), d_tab, 4 * (HTABSIZE + 1), cudaMemcpyDeviceToHost));
        ix->kmer.resize(nk);
        if (nk) ck(cudaMemcpy(ix->kmer.data(), d_kmer, 8 * nk, cudaMemcpyDeviceToHost));
        ix->strand_bits.resize((nk + 7) / 8);
        if (nk) ck(cudaMemcpy(ix->strand_bits.data(), d_bits, (nk + 7) / 8, cudaMemcpyDeviceToHost));
        unsigned long long nf = 0;
        ck(cudaMemcpy(&nf, d_nfilt, 8, cudaMemcpyDeviceToHost));
        if (nf > filt_cap) throw IbFail{FAME_ERR_INDEX};
        std::vector<ulonglong2> f(nf);
        if (nf) ck(cudaMemcpy(f.data(), d_filt, 16 * nf, cudaMemcpyDeviceToHost));
        // bucket order, then first occurrence in the bucket: the reference's scan order
        std::sort(f.begin(), f.end(), [](const ulonglong2& a, const ulonglong2& b) { return a.x < b.x; });
        std::vector<uint64_t> order(nf);
        for (uint64_t i = 0; i < nf; ++i) order[i] = f[i].y;
        index_build_finish(ix, std::move(order));
        phase("tables to the host");
    } catch (const IbFail& e) {
        delete ix;
        cudaGetLastError();
        cudaSetDevice(prev_dev);
        return e.code;
    } catch (const std::bad_alloc&) {
        delete ix;
        cudaSetDevice(prev_dev);
        return FAME_ERR_NOMEM;
    } catch (const std::exception&) {
        delete ix;
        cudaSetDevice(prev_dev);
        return FAME_ERR_NOMEM;
    }
    cudaSetDevice(prev_dev);
    *out = ix;
    return FAME_OK;
}
