// Seeding stage: spaced-seed hashes of a read, gathers from the CSR index,
// q-gram counting per window and strand, and the candidate order.
//
// Follows getSeedRefs (ReadQueue.cpp:2325-2461) and the candidate walk of
// saQuerySeedSetRef (ReadQueue.cpp:1928-2160).  FAME counts window hits in a
// per-read tsl::hopscotch_map and walks that map in its bucket order; since
// the walk order decides ties between equally good hits, this stage replays
// the map's insertions (tsl hopscotch_hash.h: power-of-two buckets, identity
// hash, 62-bucket neighbourhoods, displacement swaps, overflow list, 0.9 load
// rehash) to reproduce the order exactly.
//
// One warp handles one (read, orientation) task:
//   1. lanes hash k-mers (one k-mer per lane per step) and read tabIndex
//   2. warp prefix sum of bucket sizes; entries gathered into an op list
//   3. consecutive duplicates dropped; per (window, strand): count and first op
//      (warp __match_any_sync groups + open addressing table)
//   4. keys whose first op may insert (k-mer index <= maxQPos) listed in op order
//   5. lane 0 replays the hopscotch insertions of each map; lanes compact the
//      windows with count >= QTHRESH in bucket order (forward map first)
#pragma once
#include "dev_common.cuh"
#include "seedhash.h"

namespace fame {

constexpr uint32_t EMPTY_KEY = 0xffffffffu;
constexpr uint32_t NBHD = 62;                // hopscotch_map NeighborhoodSize
constexpr uint32_t MAX_PROBES = 12 * NBHD;   // MAX_PROBES_FOR_EMPTY_BUCKET

// Working memory of one task (shared memory for the common case, global
// scratch for reads whose bucket sizes exceed the shared-memory caps).
struct SeedMem {
    uint8_t* seq;        // oriented read, >= 256 bytes
    uint32_t* kst;       // bucket start per k-mer
    uint32_t* kpre;      // exclusive prefix of bucket sizes (nk + 1)
    uint32_t* ops;       // gathered entries
    uint8_t* opk;        // k-mer index of each op (< 256)
    uint32_t* dt_key;    // distinct (window, strand) keys
    uint32_t* dt_first;  // first op of each key; null: packed into dt_cnt (bits 0-15, ops < 65536)
    uint32_t* dt_cnt;    // count of each key (packed: bits 16-31, which wrap like the reference's uint16 count)
    uint32_t* ins;       // inserted keys, first-touch order
    uint32_t* ins_cnt;
    uint32_t* slot;      // replayed bucket array (index into ins, EMPTY_KEY if free)
    uint32_t* stk;       // pending insertions (top = next)
    uint32_t* ovf;       // overflow list
    uint32_t* stage;     // candidates of this task
    uint64_t* pre;       // prefix hashes of the read (8 * (len + 1) bytes), dead once the bucket bounds are read
    uint32_t ops_cap, dt_cap, slot_cap, stk_cap, ovf_cap;
};

__device__ __forceinline__ uint32_t pow2_ceil(uint32_t v)
{
    if (v <= 1) return 1;
    return 1u << (32 - __clz(v - 1));
}

__device__ __forceinline__ uint32_t dt_hash(uint32_t k, uint32_t mask)
{
    return (k * 0x9E3779B1u) >> 7 & mask;
}

// Replay of one map.  Returns false when a capacity is exceeded.
struct MapSim {
    uint32_t B, mask, size, nb, novf, max_thr, min_thr, sp;
};

__device__ __forceinline__ void sim_init(MapSim& m, uint32_t bucket_count)
{
    if (bucket_count > 0) {
        m.B = pow2_ceil(bucket_count);
        m.mask = m.B - 1;
        m.size = m.B + NBHD - 1;
    } else {
        m.B = 0; m.mask = 0; m.size = 0;
    }
    m.max_thr = (uint32_t)((float)m.B * 0.9f);
    m.min_thr = (uint32_t)((float)m.B * 0.1f);
}

__device__ __forceinline__ uint32_t sim_key(const SeedMem& s, uint32_t x) { return s.ins[x] & 0x7fffffffu; }

// rehash_impl (hopscotch_hash.h:1243-1300): the bucket elements are re-inserted
// in array order into a table of max(count, ceil(size / 0.9)) buckets; here they
// are pushed on the pending stack (lowest bucket on top), overflow stays.
__device__ bool sim_rehash(MapSim& m, const SeedMem& s, uint32_t count)
{
    const uint32_t need = (uint32_t)ceilf((float)m.nb / 0.9f);
    if (need > count) count = need;
    for (int b = (int)m.size - 1; b >= 0; --b) {
        const uint32_t x = s.slot[b];
        if (x != EMPTY_KEY) {
            if (m.sp >= s.stk_cap) return false;
            s.stk[m.sp++] = x;
        }
    }
    m.nb = m.novf;
    sim_init(m, count);
    if (m.size > s.slot_cap) return false;
    for (uint32_t b = 0; b < m.size; ++b) s.slot[b] = EMPTY_KEY;
    return true;
}

// insert_impl (hopscotch_hash.h:1410-1460) for the element on top of the stack.
__device__ bool sim_step(MapSim& m, const SeedMem& s)
{
    const uint32_t x = s.stk[m.sp - 1];
    const uint32_t k = sim_key(s, x);
    const uint32_t next = (m.mask + 1) * 2;
    if (m.nb - m.novf >= m.max_thr) return sim_rehash(m, s, next);
    const uint32_t ib = k & m.mask;
    // find_empty_bucket
    uint32_t ie = m.size;
    {
        const uint32_t lim = min(ib + MAX_PROBES, m.size);
        for (uint32_t b = ib; b < lim; ++b)
            if (s.slot[b] == EMPTY_KEY) { ie = b; break; }
    }
    if (ie < m.size) {
        while (true) {
            if (ie - ib < NBHD) {
                s.slot[ie] = x;
                m.nb++;
                m.sp--;
                return true;
            }
            // swap_empty_bucket_closer (hopscotch_hash.h:1541-1575)
            bool swapped = false;
            for (uint32_t tc = ie - NBHD + 1; tc < ie && !swapped; ++tc) {
                for (uint32_t ts = tc; ts < ie; ++ts) {
                    const uint32_t y = s.slot[ts];
                    if (y != EMPTY_KEY && (sim_key(s, y) & m.mask) == tc) {
                        s.slot[ie] = y;
                        s.slot[ts] = EMPTY_KEY;
                        ie = ts;
                        swapped = true;
                        break;
                    }
                }
            }
            if (!swapped) break;
        }
    }
    // will_neighborhood_change_on_rehash (hopscotch_hash.h:1465-1486)
    bool changes = false;
    const uint32_t nmask = next - 1;
    for (uint32_t b = ib; b < m.size && b - ib < NBHD; ++b) {
        const uint32_t y = s.slot[b];
        const uint32_t ky = y == EMPTY_KEY ? 0 : sim_key(s, y);
        if ((ky & m.mask) != (ky & nmask)) { changes = true; break; }
    }
    if (m.nb < m.min_thr || !changes) {
        if (m.novf >= s.ovf_cap) return false;
        s.ovf[m.novf++] = x;
        m.nb++;
        m.sp--;
        return true;
    }
    return sim_rehash(m, s, next);
}

// A warp's reservation of candidate slots: tasks take contiguous runs from
// it, so the candidate counter sees one atomic per CAND_RES_CHUNK slots
// instead of one per task.  Slots a warp reserves and leaves unused are
// marked CAND_HOLE (the window scans skip them).
constexpr uint32_t CAND_RES_CHUNK = 8;
struct CandRes {
    uint32_t base = 0, left = 0;
    uint32_t used = 0;   // slots filled since the last flush
};

__device__ __forceinline__ void cand_res_release(const ChunkBufs& cb, CandRes& res)
{
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t j = lane; j < res.left; j += 32)
        if ((uint64_t)res.base + j < cb.cand_cap) cb.cand_task[res.base + j] = CAND_HOLE;
    res.left = 0;
}

// End of a warp's tasks: unused slots become holes, the filled count is added.
__device__ __forceinline__ void cand_res_finish(const ChunkBufs& cb, CandRes& res)
{
    cand_res_release(cb, res);
    if ((threadIdx.x & 31) == 0 && res.used) atomicAdd(cb.ctr + CTR_CAND_USED, (unsigned long long)res.used);
    res.used = 0;
}

// Warp-cooperative seeding of one task.  Returns 0 on success, 1 when the task
// does not fit the memory caps (the caller hands it to the heavy path).
// All lanes of the warp must call it.
__device__ int seed_task(const DevIndex& ix, const ChunkBufs& cb, const SeedMem& s, uint32_t task,
                         unsigned long long* gather_bytes_acc, CandRes& res)
{
    const int lane = threadIdx.x & 31;
    const uint32_t r = task >> 1, o = task & 1;
    const uint64_t off0 = cb.offs[r];
    const uint32_t len = (uint32_t)(cb.offs[r + 1] - off0);
    const char* raw = cb.seqs + off0;
    for (uint32_t p = lane; p < len; p += 32) {
        const uint8_t c = (uint8_t)raw[p];
        if (o == 0) s.seq[p] = c;
        else s.seq[len - 1 - p] = rc_byte(c);
    }
    __syncwarp();
    // 1. hashes and bucket bounds (getSeedRefs pass 1, ReadQueue.cpp:2331-2354):
    //    every lane first hashes its k-mers, then issues all of its bucket
    //    reads before using any, so their DRAM latencies overlap.  Hashes by
    //    the prefix form of seedhash.h: P[j] (j <= len, 8 bytes each) in an
    //    area that is dead until the gather or the count.
    const uint32_t nk = len - KMERLEN + 1;
    uint32_t sigma = 0;
    unsigned long long gb = 0;
    uint64_t* P = s.pre;
    {
        uint64_t carry = 0;   // P[b]
        for (uint32_t b = 0; b <= len; b += 32) {
            const uint32_t j = b + lane;
            const uint64_t u = j < len ? sh_u(s.seq[j], j) : 0ull;
            uint64_t inc = u;   // u[b] ^ ... ^ u[j]
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint64_t t = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= (uint32_t)d) inc ^= t;
            }
            if (j <= len) P[j] = carry ^ inc ^ u;
            carry ^= __shfl_sync(0xffffffffu, inc, 31);
        }
    }
    __syncwarp();
    for (uint32_t p = lane; p < nk; p += 32) s.kst[p] = sh_prefix_hash([&](uint32_t j) { return P[j]; }, p, HTAB_MASK);
    constexpr int KPL = (FAME_MAX_READ_LEN - KMERLEN + 1 + 31) / 32;   // k-mers per lane, at most
    uint32_t e0[KPL];                                                    // first entry of each bucket
    {
        uint32_t b0[KPL], b1[KPL];
#pragma unroll
        for (int j = 0; j < KPL; ++j) {
            const uint32_t p = lane + 32 * j;
            if (p < nk) {
                const uint32_t key = s.kst[p];
                const uint2 t = __ldg(ix.tab2 + key);
                b0[j] = t.x;
                e0[j] = t.y;
                b1[j] = __ldg((const uint32_t*)(ix.tab2 + key + 1));
            }
        }
#pragma unroll
        for (int j = 0; j < KPL; ++j) {
            const uint32_t p = lane + 32 * j;
            if (p < nk) {
                s.kst[p] = b0[j];
                s.kpre[p] = b1[j] - b0[j];
                sigma += b1[j] - b0[j];
                gb += 8 + 4ull * (b1[j] - b0[j]);
            }
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        sigma += __shfl_xor_sync(0xffffffffu, sigma, d);
        gb += __shfl_xor_sync(0xffffffffu, gb, d);
    }
    __syncwarp();
    // exclusive prefix of bucket sizes over k-mers (contiguous chunk per lane)
    {
        const uint32_t per = (nk + 31) / 32;
        const uint32_t b = min(nk, lane * per), e = min(nk, b + per);
        uint32_t loc = 0;
        for (uint32_t p = b; p < e; ++p) loc += s.kpre[p];
        uint32_t inc = loc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += v;
        }
        uint32_t run = inc - loc;
        __syncwarp();
        for (uint32_t p = b; p < e; ++p) { const uint32_t l = s.kpre[p]; s.kpre[p] = run; run += l; }
        if (lane == 31) s.kpre[nk] = inc;
    }
    __syncwarp();
    const uint32_t T = s.kpre[nk];
    if (T > s.ops_cap) return 1;
    if (lane == 0) atomicAdd(gather_bytes_acc, gb);
    // 2. gather entries (getSeedRefs pass 2, ReadQueue.cpp:2361-2460): the
    //    first entry of each bucket came with its bounds; the k-mer of every
    //    op, then the other entries, up to 8 reads per lane in flight
#pragma unroll
    for (int j = 0; j < KPL; ++j) {
        const uint32_t p = lane + 32 * j;
        if (p < nk && s.kpre[p + 1] > s.kpre[p]) s.ops[s.kpre[p]] = e0[j];
    }
    for (uint32_t p = lane; p < nk; p += 32) {
        const uint32_t b = s.kpre[p], n = s.kpre[p + 1] - b;
        for (uint32_t j = 0; j < n; ++j) s.opk[b + j] = (uint8_t)p;
    }
    __syncwarp();
    for (uint32_t base = 0; base < T; base += 256) {
        uint32_t e[8];
        bool ld[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = base + lane + 32 * j;
            ld[j] = false;
            if (i < T) {
                const uint32_t p = s.opk[i];
                const uint32_t k = i - s.kpre[p];
                if (k > 0) {
                    e[j] = __ldg(ix.entry + s.kst[p] + k);
                    ld[j] = true;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = base + lane + 32 * j;
            if (ld[j]) s.ops[i] = e[j];
        }
    }
    // 3. distinct keys with counts and first op (consecutive duplicates within a
    //    bucket are skipped, ReadQueue.cpp:2380-2387, 2421-2428)
    const uint32_t dsz = min(s.dt_cap, pow2_ceil(2 * T + 2));
    const uint32_t dmask = dsz - 1;
    const bool packed = s.dt_first == nullptr;
    const uint32_t cnt_shift = packed ? 16 : 0;
    for (uint32_t i = lane; i < dsz; i += 32) s.dt_key[i] = EMPTY_KEY;
    __syncwarp();
    for (uint32_t b0 = 0; b0 < T; b0 += 32) {
        const uint32_t i = b0 + lane;
        bool valid = false;
        uint32_t e = 0;
        if (i < T) {
            e = s.ops[i];
            valid = !(i > s.kpre[s.opk[i]] && s.ops[i - 1] == e);
        }
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        const unsigned grp = __match_any_sync(0xffffffffu, valid ? e : EMPTY_KEY) & vm;
        if (valid && (__ffs(grp) - 1) == lane) {
            uint32_t h = dt_hash(e, dmask);
            while (true) {
                const uint32_t cur = s.dt_key[h];
                if (cur == e) break;
                if (cur == EMPTY_KEY) {
                    const uint32_t old = atomicCAS(&s.dt_key[h], EMPTY_KEY, e);
                    if (old == EMPTY_KEY) {
                        if (packed) s.dt_cnt[h] = i;
                        else { s.dt_first[h] = i; s.dt_cnt[h] = 0; }
                        break;
                    }
                    if (old == e) break;
                }
                h = (h + 1) & dmask;
            }
            s.dt_cnt[h] += (uint32_t)__popc(grp) << cnt_shift;
        }
        __syncwarp();
    }
    // 4. inserted keys in first-touch order: the first op of a key inserts iff
    //    its k-mer is the first one or cIdx < maxQPos (ReadQueue.cpp:2371, 2430)
    const uint32_t maxQPos = len - KMERLEN + 1 - QTHRESH;
    uint32_t nins = 0;
    for (uint32_t b0 = 0; b0 < T; b0 += 32) {
        const uint32_t i = b0 + lane;
        bool take = false;
        uint32_t e = 0, c = 0;
        if (i < T) {
            e = s.ops[i];
            const uint32_t k = s.opk[i];
            if (!(i > s.kpre[k] && s.ops[i - 1] == e) && (k == 0 || k - 1 < maxQPos)) {
                uint32_t h = dt_hash(e, dmask);
                while (s.dt_key[h] != e) h = (h + 1) & dmask;
                const uint32_t v = s.dt_cnt[h];
                if ((packed ? (v & 0xffffu) : s.dt_first[h]) == i) { take = true; c = v >> cnt_shift; }
            }
        }
        const unsigned bm = __ballot_sync(0xffffffffu, take);
        if (take) {
            const uint32_t at = nins + __popc(bm & ((1u << lane) - 1));
            s.ins[at] = e;
            s.ins_cnt[at] = c;
        }
        nins += __popc(bm);
        __syncwarp();
    }
    // 5. replay both maps (forward map first, the order saQuerySeedSetRef walks)
    //    on lane 0; the ops/dt memory is dead from here and may alias slot/stk/ovf
    uint32_t nstage = 0, nf = 0;
    bool fail = false;
    for (int dir = 1; dir >= 0; --dir) {
        // A map with at most one candidate (count >= QTHRESH) needs no replay:
        // its walk sees that candidate alone, wherever the other keys sit.
        uint32_t ndc = 0, only = 0;
        for (uint32_t b0 = 0; b0 < nins; b0 += 32) {
            const uint32_t x = b0 + lane;
            const uint32_t v = x < nins ? s.ins[x] : 0u;
            const bool take = x < nins && (v >> 31) == (uint32_t)dir && (s.ins_cnt[x] & 0xffffu) >= QTHRESH;
            const unsigned bm = __ballot_sync(0xffffffffu, take);
            if (bm) {
                const uint32_t first = __shfl_sync(0xffffffffu, v, __ffs(bm) - 1);
                if (ndc == 0) only = first;
            }
            ndc += __popc(bm);
        }
        if (ndc <= 1) {
            if (ndc == 1 && lane == 0) s.stage[nstage] = only;
            nstage += ndc;
            __syncwarp();
            if (dir == 1) nf = nstage;
            continue;
        }
        MapSim m;
        sim_init(m, sigma / 5);
        m.nb = 0; m.novf = 0; m.sp = 0;
        if (m.size > s.slot_cap) { fail = true; }
        if (!__any_sync(0xffffffffu, fail)) {
            for (uint32_t b = lane; b < m.size; b += 32) s.slot[b] = EMPTY_KEY;
            __syncwarp();
            if (lane == 0) {
                for (uint32_t x = 0; x < nins && !fail; ++x) {
                    if ((s.ins[x] >> 31) != (uint32_t)dir) continue;
                    if (m.sp >= s.stk_cap) { fail = true; break; }
                    s.stk[m.sp++] = x;
                    while (m.sp > 0) {
                        if (!sim_step(m, s)) { fail = true; break; }
                    }
                }
            }
            fail = __shfl_sync(0xffffffffu, fail, 0);
            m.size = __shfl_sync(0xffffffffu, m.size, 0);
            m.novf = __shfl_sync(0xffffffffu, m.novf, 0);
            __syncwarp();
        }
        if (fail) break;
        // iteration order: buckets in array order, then the overflow list
        for (uint32_t b0 = 0; b0 < m.size + m.novf; b0 += 32) {
            const uint32_t b = b0 + lane;
            uint32_t x = EMPTY_KEY;
            if (b < m.size) x = s.slot[b];
            else if (b < m.size + m.novf) x = s.ovf[b - m.size];
            const bool take = x != EMPTY_KEY && (s.ins_cnt[x] & 0xffffu) >= QTHRESH;
            const unsigned bm = __ballot_sync(0xffffffffu, take);
            if (take) s.stage[nstage + __popc(bm & ((1u << lane) - 1))] = s.ins[x];
            nstage += __popc(bm);
        }
        __syncwarp();
        if (dir == 1) nf = nstage;
    }
    if (fail) return 1;
    // 6. publish the candidates, contiguous, from the warp's reservation
    uint32_t base = 0;
    if (nstage) {
        if (nstage > res.left) {
            cand_res_release(cb, res);
            const uint32_t want = max(nstage, CAND_RES_CHUNK);
            if (lane == 0) res.base = (uint32_t)atomicAdd(cb.ctr + CTR_CAND, (unsigned long long)want);
            res.base = __shfl_sync(0xffffffffu, res.base, 0);
            res.left = want;
        }
        base = res.base;
        res.base += nstage;
        res.left -= nstage;
        res.used += nstage;
    }
    if ((uint64_t)base + nstage <= cb.cand_cap) {
        for (uint32_t j = lane; j < nstage; j += 32) {
            cb.cand[base + j] = s.stage[j];
            cb.cand_task[base + j] = task;
        }
    }
    if (lane == 0) cb.task_cand[task] = make_uint4(base, nf, nstage - nf, 0);
    return 0;
}

}  // namespace fame
