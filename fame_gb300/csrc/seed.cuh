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
//   2. warp prefix sum of bucket sizes; entries gathered in op order
//   3. as they arrive: consecutive duplicates dropped; per (window, strand):
//      count and first op (warp __match_any_sync groups + open addressing
//      table), the keys whose count reaches QTHRESH noted
//   4. when neither strand map has two candidates (the common case) the
//      candidates are staged at once; otherwise the keys whose first op may
//      insert (k-mer index <= maxQPos) are listed in op order and
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

// The same replay run by a whole warp (every lane calls with the same state;
// the state stays warp-uniform).  Scans of up to 62 buckets take one or two
// warp steps instead of a loop per bucket; lane 0 writes the buckets and
// the stack, and a __syncwarp orders every write before the next read.

__device__ __forceinline__ uint32_t warp_min_u32(uint32_t v)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, d));
    return v;
}

// rehash_impl: the bucket elements pushed in descending bucket order (so the
// lowest bucket ends on top of the stack), the overflow list kept.
__device__ bool sim_rehash_w(MapSim& m, const SeedMem& s, uint32_t count)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t need = (uint32_t)ceilf((float)m.nb / 0.9f);
    if (need > count) count = need;
    uint32_t sp = m.sp;
    for (uint32_t top = m.size; top > 0; top = top > 32 ? top - 32 : 0) {
        const int b = (int)top - 1 - (int)lane;   // lane 0 takes the highest bucket of this step
        const uint32_t x = b >= 0 ? s.slot[b] : EMPTY_KEY;
        const unsigned bm = __ballot_sync(0xffffffffu, x != EMPTY_KEY);
        if (sp + __popc(bm) > s.stk_cap) return false;
        if (x != EMPTY_KEY) s.stk[sp + __popc(bm & ((1u << lane) - 1))] = x;
        sp += __popc(bm);
    }
    m.sp = sp;
    m.nb = m.novf;
    sim_init(m, count);
    __syncwarp();
    if (m.size > s.slot_cap) return false;
    for (uint32_t b = lane; b < m.size; b += 32) s.slot[b] = EMPTY_KEY;
    __syncwarp();
    return true;
}

// insert_impl for the element on top of the stack.
__device__ bool sim_step_w(MapSim& m, const SeedMem& s)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t x = s.stk[m.sp - 1];
    const uint32_t k = sim_key(s, x);
    const uint32_t next = (m.mask + 1) * 2;
    if (m.nb - m.novf >= m.max_thr) return sim_rehash_w(m, s, next);
    const uint32_t ib = k & m.mask;
    // find_empty_bucket: the first empty bucket in [ib, ib + MAX_PROBES)
    uint32_t ie = m.size;
    {
        const uint32_t lim = min(ib + MAX_PROBES, m.size);
        for (uint32_t b0 = ib; b0 < lim; b0 += 32) {
            const uint32_t b = b0 + lane;
            const unsigned em = __ballot_sync(0xffffffffu, b < lim && s.slot[b] == EMPTY_KEY);
            if (em) { ie = b0 + __ffs(em) - 1; break; }
        }
    }
    if (ie < m.size) {
        while (true) {
            if (ie - ib < NBHD) {
                if (lane == 0) s.slot[ie] = x;
                m.nb++;
                m.sp--;
                __syncwarp();
                return true;
            }
            // swap_empty_bucket_closer: of the elements at ts in [ie - NBHD + 1, ie)
            // whose home bucket tc lies in [ie - NBHD + 1, ts], the one with the
            // smallest tc, then the smallest ts, moves to ie
            const uint32_t lo = ie - NBHD + 1;
            uint32_t best = 0xffffffffu;
            for (uint32_t t0 = lo; t0 < ie; t0 += 32) {
                const uint32_t ts = t0 + lane;
                if (ts < ie) {
                    const uint32_t y = s.slot[ts];
                    if (y != EMPTY_KEY) {
                        const uint32_t tc = sim_key(s, y) & m.mask;
                        if (tc >= lo && tc <= ts) best = min(best, ((tc - lo) << 8) | (ts - lo));
                    }
                }
            }
            best = warp_min_u32(best);
            if (best == 0xffffffffu) break;
            const uint32_t ts = lo + (best & 0xffu);
            if (lane == 0) {
                s.slot[ie] = s.slot[ts];
                s.slot[ts] = EMPTY_KEY;
            }
            __syncwarp();
            ie = ts;
        }
    }
    // will_neighborhood_change_on_rehash
    const uint32_t nmask = next - 1;
    bool changes = false;
    {
        const uint32_t lim = min(m.size, ib + NBHD);
        for (uint32_t b0 = ib; b0 < lim && !changes; b0 += 32) {
            const uint32_t b = b0 + lane;
            bool ch = false;
            if (b < lim) {
                const uint32_t y = s.slot[b];
                const uint32_t ky = y == EMPTY_KEY ? 0 : sim_key(s, y);
                ch = (ky & m.mask) != (ky & nmask);
            }
            changes = __any_sync(0xffffffffu, ch);
        }
    }
    if (m.nb < m.min_thr || !changes) {
        if (m.novf >= s.ovf_cap) return false;
        if (lane == 0) s.ovf[m.novf] = x;
        m.novf++;
        m.nb++;
        m.sp--;
        __syncwarp();
        return true;
    }
    return sim_rehash_w(m, s, next);
}

// Runs insert_impl for the elements on the stack until it is empty, up to
// 32 at a time: the top elements are tried at once (lane k the k-th from
// the top); an element whose first empty bucket from its home lies in its
// neighbourhood, that no element above it wants too, and that keeps the load
// under the rehash threshold is placed exactly where one insert_impl after
// another would place it.  The elements above the first one that fails these
// tests go in together, and that one (then on top) runs the full insert_impl
// (displacements, overflow list, or a rehash that pushes the table's
// elements on top of the stack, which the next steps drain the same way).
// False when a cap is exceeded.
__device__ bool sim_drain_w(MapSim& m, const SeedMem& s)
{
    constexpr uint32_t FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31;
    while (m.sp > 0) {
        const uint32_t n = min(32u, m.sp);
        const bool act = lane < n;
        const uint32_t x = act ? s.stk[m.sp - 1 - lane] : 0u;
        uint32_t ie = m.size;
        bool ok = false;
        if (act && m.size > 0) {
            const uint32_t ib = sim_key(s, x) & m.mask;
            const uint32_t lim = min(ib + MAX_PROBES, m.size);
            for (uint32_t b = ib; b < lim; ++b)
                if (s.slot[b] == EMPTY_KEY) { ie = b; break; }
            ok = ie < m.size && ie - ib < NBHD && m.nb + lane - m.novf < m.max_thr;
        }
        // an element that wants a bucket an element above it wants too fails
        const unsigned grp = __match_any_sync(FULL, act ? ie : 0xfffffff0u - lane);
        if (act && (uint32_t)(__ffs(grp) - 1) != lane) ok = false;
        const unsigned bad = __ballot_sync(FULL, act && !ok);
        const uint32_t ngood = bad ? (uint32_t)(__ffs(bad) - 1) : n;
        if (lane < ngood) s.slot[ie] = x;
        m.nb += ngood;
        m.sp -= ngood;
        __syncwarp();
        if (bad && !sim_step_w(m, s)) return false;
    }
    return true;
}

// Inserts, in lane order, the keys ins[xb + lane] of the lanes in `todo`
// (the stack empty on entry and on return): they go on the stack, the first
// on top, and the stack is drained.  False when a cap is exceeded.
__device__ bool sim_insert_batch_w(MapSim& m, const SeedMem& s, uint32_t xb, unsigned todo)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t k = __popc(todo);
    if (m.sp + k > s.stk_cap) return false;
    if ((todo >> lane) & 1u) s.stk[m.sp + k - 1 - __popc(todo & ((1u << lane) - 1))] = xb + lane;
    m.sp += k;
    __syncwarp();
    return sim_drain_w(m, s);
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

// Publishes a task's candidates (stage[0 .. nstage), the first nf from the
// forward map), contiguous, from the warp's slot reservation.
__device__ __forceinline__ void seed_publish(const ChunkBufs& cb, CandRes& res, uint32_t task, const uint32_t* stage,
                                             uint32_t nstage, uint32_t nf)
{
    const uint32_t lane = threadIdx.x & 31;
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
            cb.cand[base + j] = stage[j];
            cb.cand_task[base + j] = task;
        }
    }
    if (lane == 0) cb.task_cand[task] = make_uint4(base, nf, nstage - nf, 0);
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
                uint32_t slot;
                const uint4 t = rec_lookup(ix, s.kst[p], slot);
                b0[j] = t.x;
                e0[j] = t.z;
                b1[j] = t.x + t.y;
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
    // the count table (the prefix hashes that may share its memory are dead)
    const uint32_t dsz = min(s.dt_cap, pow2_ceil(2 * T + 2));
    const uint32_t dmask = dsz - 1;
    const bool packed = s.dt_first == nullptr;
    const uint32_t cnt_shift = packed ? 16 : 0;
    for (uint32_t i = lane; i < dsz; i += 32) s.dt_key[i] = EMPTY_KEY;
    // keys whose count reached QTHRESH, by count-table slot (in the memory of
    // the inserted keys, which are listed later and only when needed)
    uint32_t* reached = s.ins;
    const uint32_t reached_cap = min(32u, s.ops_cap);
    uint32_t nreached = 0;
    __syncwarp();
    // 3. count the distinct keys as their entries arrive, with each key's
    //    first op (consecutive duplicates within a bucket are skipped,
    //    ReadQueue.cpp:2380-2387, 2421-2428): ops in order, 32 at a time;
    //    an op's predecessor is the previous lane's entry (lane 0: lane 31's
    //    of the step before)
    uint32_t last = EMPTY_KEY;
    for (uint32_t base = 0; base < T; base += 256) {
        uint32_t e[8];
        bool inner[8];   // not the first entry of its bucket
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = base + lane + 32 * j;
            e[j] = EMPTY_KEY;
            inner[j] = false;
            if (i < T) {
                const uint32_t p = s.opk[i];
                const uint32_t k = i - s.kpre[p];
                inner[j] = k > 0;
                e[j] = k > 0 ? __ldg(ix.entry + s.kst[p] + k) : s.ops[i];
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = base + lane + 32 * j;
            if (inner[j]) s.ops[i] = e[j];
            uint32_t prev = __shfl_up_sync(0xffffffffu, e[j], 1);
            if (lane == 0) prev = last;
            last = __shfl_sync(0xffffffffu, e[j], 31);
            const bool valid = i < T && !(inner[j] && prev == e[j]);
            const unsigned vm = __ballot_sync(0xffffffffu, valid);
            const unsigned grp = __match_any_sync(0xffffffffu, valid ? e[j] : EMPTY_KEY) & vm;
            bool reach = false;
            uint32_t h = 0;
            if (valid && (__ffs(grp) - 1) == lane) {
                const uint32_t key = e[j];
                h = dt_hash(key, dmask);
                while (true) {
                    const uint32_t cur = s.dt_key[h];
                    if (cur == key) break;
                    if (cur == EMPTY_KEY) {
                        const uint32_t old = atomicCAS(&s.dt_key[h], EMPTY_KEY, key);
                        if (old == EMPTY_KEY) {
                            if (packed) s.dt_cnt[h] = i;
                            else { s.dt_first[h] = i; s.dt_cnt[h] = 0; }
                            break;
                        }
                        if (old == key) break;
                    }
                    h = (h + 1) & dmask;
                }
                const uint32_t before = s.dt_cnt[h] >> cnt_shift;
                const uint32_t add = (uint32_t)__popc(grp);
                s.dt_cnt[h] += add << cnt_shift;
                reach = before < QTHRESH && before + add >= QTHRESH;
            }
            const unsigned rm = __ballot_sync(0xffffffffu, reach);
            if (reach) {
                const uint32_t at = nreached + __popc(rm & ((1u << lane) - 1));
                if (at < reached_cap) reached[at] = h;
            }
            nreached += __popc(rm);
            __syncwarp();   // this op's count-table writes before the next op's probes
        }
    }
    const uint32_t maxQPos = len - KMERLEN + 1 - QTHRESH;
    uint32_t nstage = 0, nf = 0;
    // 4. the candidates (keys inserted into the map, ReadQueue.cpp:2371, 2430:
    //    their first op's k-mer is the first one or cIdx < maxQPos; with a
    //    count >= QTHRESH).  A strand map with at most one candidate needs no
    //    insertion order: its walk sees that candidate alone, wherever the
    //    other keys sit.  When both maps have at most one, they are staged
    //    at once (forward map first, the order saQuerySeedSetRef walks).
    //    Counts stay below 65536 here, so no uint16 wrap can hide a crossing.
    bool ordered = false;
    if (T < 65536 && nreached <= reached_cap) {
        uint32_t key = 0;
        bool cand = false;
        if (lane < nreached) {
            const uint32_t h = reached[lane];
            const uint32_t first = packed ? (s.dt_cnt[h] & 0xffffu) : s.dt_first[h];
            const uint32_t k = s.opk[first];
            cand = k == 0 || k - 1 < maxQPos;
            key = s.dt_key[h];
        }
        const unsigned fm = __ballot_sync(0xffffffffu, cand && (key >> 31));
        const unsigned bm = __ballot_sync(0xffffffffu, cand && !(key >> 31));
        if (__popc(fm) <= 1 && __popc(bm) <= 1) {
            nf = __popc(fm);
            nstage = nf + __popc(bm);
            if (cand) s.stage[(key >> 31) ? 0 : nf] = key;
            ordered = true;
        }
    }
    __syncwarp();
    if (!ordered) {
        if (lane == 0) atomicAdd(cb.ctr + CTR_REPLAY, 1ull);
        // 4b. inserted keys in first-touch order: the first op of a key
        //     inserts iff its k-mer is the first one or cIdx < maxQPos
        //     (ReadQueue.cpp:2371, 2430)
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
        // 5. replay both maps (forward map first, the order saQuerySeedSetRef
        //    walks) on lane 0; the ops/dt memory is dead from here and may
        //    alias slot/stk/ovf
        bool fail = false;
        for (int dir = 1; dir >= 0; --dir) {
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
            if (!fail) {
                for (uint32_t b = lane; b < m.size; b += 32) s.slot[b] = EMPTY_KEY;
                __syncwarp();
                // this map's keys in first-touch order, each inserted by the warp
                for (uint32_t b0 = 0; b0 < nins && !fail; b0 += 32) {
                    const uint32_t xl = b0 + lane;
                    unsigned todo = __ballot_sync(0xffffffffu, xl < nins && (s.ins[xl] >> 31) == (uint32_t)dir);
                    while (todo && !fail) {
                        const uint32_t x = b0 + __ffs(todo) - 1;
                        todo &= todo - 1;
                        if (m.sp >= s.stk_cap) { fail = true; break; }
                        if (lane == 0) s.stk[m.sp] = x;
                        m.sp++;
                        __syncwarp();
                        while (m.sp > 0) {
                            if (!sim_step_w(m, s)) { fail = true; break; }
                        }
                    }
                }
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
    }
    // 6. publish the candidates
    seed_publish(cb, res, task, s.stage, nstage, nf);
    return 0;
}

// ---------------------------------------------------------------------------
// Seeding from the bucket records (the light and middle tiers): the same
// results as seed_task with less memory traffic and working memory.
//
// Each lane owns k-mers (p = lane + 32 jj).  A k-mer's record (one aligned
// sector) gives its bucket's bounds and first REC_INLINE entries, so for
// most buckets one DRAM line serves the whole lookup; longer buckets stream
// the rest of their entries from the entry table, each load issued
// REC_INLINE entries before its use.  The count needs no order: sub-step j
// takes entry j of every lane's bucket, skipping an entry equal to its
// predecessor in the bucket (consecutive duplicates, ReadQueue.cpp:2380-2387,
// 2421-2428), and the lanes that hold one key add their ops through one
// leader (warp match groups).  A key is inserted into the
// map (ReadQueue.cpp:2371, 2430) iff its first op's k-mer index is at most
// maxQPos; ops come in k-mer order, so that holds iff some op of the key has
// such an index, i.e. iff the key's count exceeds its count of ops from the
// k-mers past maxQPos.  The same word keeps the dense index of the key's
// first op (ops ordered by k-mer, then entry: within a sub-step the group's
// leader, the lowest lane, holds the first), so when a strand map has two or
// more candidates the insertion order the map replay needs is a rank of the
// inserted keys by first op, through a bitmap.
// ---------------------------------------------------------------------------
struct SeedMemR {
    uint8_t* seq;        // oriented read, 256 bytes
    uint64_t* pre;       // prefix hashes (aliases the count table)
    uint16_t* ksz;       // bucket size per k-mer
    uint32_t* kpre;      // exclusive prefix of bucket sizes (nk + 1), for the replay order
    uint32_t* dt_key;    // count table: distinct (window, strand) keys
    uint32_t* dt_val;    //   count | count of ops past maxQPos << 10 | first op << 20
    uint32_t* reached;   // [0, 32) count-table slots whose count reached QTHRESH,
                         // [33, 35) the staged candidates of the common case
    uint32_t* bitmap;    // one bit per op (1024 bits): the first ops of the inserted keys (replay only)
    uint32_t* ins;       // inserted keys in first-touch order (replay only)
    uint16_t* ins_cnt;   //   and their counts
    uint32_t* slot;      // replayed buckets, pending stack, overflow list and the
    uint32_t* stk;       // staged candidates: over the dead per-k-mer arrays and
    uint32_t* ovf;       // count table once the insertion order is listed
    uint32_t* stage;
    uint32_t ops_cap, dt_cap, slot_cap, stk_cap, ovf_cap;
};

// count-table word: count (bits 0-9), count of ops from k-mers past maxQPos
// (bits 10-19), dense index of the key's first op (bits 20-29; 1023 before
// any), for at most 1023 gathered entries
constexpr uint32_t DTV_TAIL = 1u << 10;
constexpr uint32_t DTV_FIRST_SHIFT = 20;
constexpr uint32_t DTV_EMPTY = 1023u << DTV_FIRST_SHIFT;
__device__ __forceinline__ uint32_t dtv_count(uint32_t v) { return v & 1023u; }
__device__ __forceinline__ uint32_t dtv_first(uint32_t v) { return (v >> DTV_FIRST_SHIFT) & 1023u; }
__device__ __forceinline__ bool dtv_inserted(uint32_t v) { return dtv_count(v) > ((v >> 10) & 1023u); }

// Shared-memory working set of one warp for seed_task_rec: up to OPS
// gathered bucket entries, a DT-slot count table (a power of two >= 2 * OPS).
// The per-k-mer arrays, the count table (prefix hashes first) and, once the
// insertion order is listed, the replay's buckets, stack, overflow list and
// staged candidates share one region.
template <uint32_t OPS, uint32_t DT, uint32_t OVF_N>
struct SeedLayoutR {
    static_assert(DT >= 2 * OPS && (DT & (DT - 1)) == 0 && OPS < 1024, "count table too small");
    static constexpr uint32_t R16(uint32_t b) { return (b + 15) / 16 * 16; }
    static constexpr uint32_t SLOT_N = DT + 64;    // replayed buckets: pow2_ceil(OPS + 1) + 61 at most
    static constexpr uint32_t SEQ = 0;             // 256 B
    static constexpr uint32_t KSZ = SEQ + 256;     // 224 x u16
    static constexpr uint32_t KPRE = KSZ + 448;    // 225 x u32
    static constexpr uint32_t DTK = KPRE + 912;
    static constexpr uint32_t DTV = DTK + DT * 4;
    static constexpr uint32_t END_U = DTV + DT * 4;
    static constexpr uint32_t BITMAP = END_U;      // 32 x u32
    static constexpr uint32_t REACHED = BITMAP + 128; // 36 x u32
    static constexpr uint32_t INS = REACHED + 144;
    static constexpr uint32_t INSC = INS + R16(OPS * 4);
    static constexpr uint32_t BYTES = INSC + R16(OPS * 2);
    // the replay, over [0, END_U)
    static constexpr uint32_t SLOT = 0;
    static constexpr uint32_t STK = SLOT + R16(SLOT_N * 4);
    static constexpr uint32_t OVF = STK + R16(OPS * 4);
    static constexpr uint32_t STAGE = OVF + R16(OVF_N * 4);
    static constexpr uint32_t END_B = STAGE + R16(OPS * 4);
    static_assert(END_B <= END_U, "the replay does not fit the shared region");
    static_assert(DTK % 8 == 0 && END_U - DTK >= 8 * (FAME_MAX_READ_LEN + 1), "prefix hashes do not fit");
};

template <class L, uint32_t OPS, uint32_t DT, uint32_t OVF_N>
__device__ __forceinline__ SeedMemR seed_mem_r(uint8_t* base)
{
    SeedMemR s;
    s.seq = base + L::SEQ;
    s.ksz = (uint16_t*)(base + L::KSZ);
    s.kpre = (uint32_t*)(base + L::KPRE);
    s.bitmap = (uint32_t*)(base + L::BITMAP);
    s.pre = (uint64_t*)(base + L::DTK);
    s.dt_key = (uint32_t*)(base + L::DTK);
    s.dt_val = (uint32_t*)(base + L::DTV);
    s.reached = (uint32_t*)(base + L::REACHED);
    s.ins = (uint32_t*)(base + L::INS);
    s.ins_cnt = (uint16_t*)(base + L::INSC);
    s.slot = (uint32_t*)(base + L::SLOT);
    s.stk = (uint32_t*)(base + L::STK);
    s.ovf = (uint32_t*)(base + L::OVF);
    s.stage = (uint32_t*)(base + L::STAGE);
    s.ops_cap = OPS; s.dt_cap = DT; s.slot_cap = L::SLOT_N; s.stk_cap = OPS; s.ovf_cap = OVF_N;
    return s;
}

template <class L, uint32_t OPS, uint32_t DT, uint32_t OVF_N>
__device__ __noinline__ int seed_rec_replay(uint8_t* base, unsigned long long* ctr, uint32_t T);

// base: the warp's working memory (layout L).  Returns 0 when the task's
// candidates are published, 1 when the task is over the caps.
template <class L, uint32_t OPS, uint32_t DT, uint32_t OVF_N>
__device__ __forceinline__ int seed_task_rec(const DevIndex& ix, const ChunkBufs& cb, uint8_t* base, uint32_t task,
                                             unsigned long long* gather_bytes_acc, CandRes& res)
{
    const SeedMemR s = seed_mem_r<L, OPS, DT, OVF_N>(base);
    constexpr uint32_t FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31;
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
    // 1. hashes (getSeedRefs pass 1, ReadQueue.cpp:2331-2354) by the prefix
    //    form of seedhash.h, then every lane's record loads before any use
    const uint32_t nk = len - KMERLEN + 1;
    uint64_t* P = s.pre;
    {
        uint64_t carry = 0;
        for (uint32_t b = 0; b <= len; b += 32) {
            const uint32_t j = b + lane;
            const uint64_t u = j < len ? sh_u(s.seq[j], j) : 0ull;
            uint64_t inc = u;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint64_t t = __shfl_up_sync(FULL, inc, d);
                if (lane >= (uint32_t)d) inc ^= t;
            }
            if (j <= len) P[j] = carry ^ inc ^ u;
            carry ^= __shfl_sync(FULL, inc, 31);
        }
    }
    __syncwarp();
    constexpr int KPL = (FAME_MAX_READ_LEN - KMERLEN + 1 + 31) / 32;   // k-mers per lane, at most
    uint32_t key[KPL];
    uint4 lo[KPL];     // {start, size, e0, e1}
#pragma unroll
    for (int jj = 0; jj < KPL; ++jj) {
        const uint32_t p = lane + 32 * jj;
        key[jj] = p < nk ? sh_prefix_hash([&](uint32_t j) { return P[j]; }, p, HTAB_MASK) : 0u;
    }
    if (!ix.rec_hashed) {
#pragma unroll
        for (int jj = 0; jj < KPL; ++jj) {
            const uint32_t p = lane + 32 * jj;
            lo[jj] = p < nk ? __ldg(ix.rec + 2ull * key[jj]) : make_uint4(0, 0, 0, 0);
        }
    } else {
        // hashed records (small genomes): probe, then keep the slot where the key was
#pragma unroll
        for (int jj = 0; jj < KPL; ++jj) {
            const uint32_t p = lane + 32 * jj;
            uint32_t slot = 0;
            lo[jj] = p < nk ? rec_lookup(ix, key[jj], slot) : make_uint4(0, 0, 0, 0);
            key[jj] = slot;
        }
    }
    __syncwarp();   // the prefix hashes are dead: the count table may take their memory
    for (uint32_t i = lane; i < DT; i += 32) {
        s.dt_key[i] = EMPTY_KEY;
        s.dt_val[i] = DTV_EMPTY;
    }
    uint32_t T = 0;
    unsigned long long gb = 0;
#pragma unroll
    for (int jj = 0; jj < KPL; ++jj) {
        const uint32_t p = lane + 32 * jj;
        if (p < nk) {
            s.ksz[p] = (uint16_t)lo[jj].y;
            T += lo[jj].y;
            gb += 8 + 4ull * lo[jj].y;
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        T += __shfl_xor_sync(FULL, T, d);
        gb += __shfl_xor_sync(FULL, gb, d);
    }
    if (T > OPS) return 1;
    if (lane == 0) atomicAdd(gather_bytes_acc, gb);
    const uint32_t maxQPos = len - KMERLEN + 1 - QTHRESH;
    uint32_t nreached = 0;
    __syncwarp();
    // dense op index of each k-mer's first entry: exclusive prefix of the bucket sizes
    {
        const uint32_t per = (nk + 31) / 32;
        const uint32_t b = min(nk, lane * per), e = min(nk, b + per);
        uint32_t loc = 0;
        for (uint32_t p = b; p < e; ++p) loc += s.ksz[p];
        uint32_t inc = loc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, inc, d);
            if (lane >= (uint32_t)d) inc += t;
        }
        uint32_t run = inc - loc;
        for (uint32_t p = b; p < e; ++p) { s.kpre[p] = run; run += s.ksz[p]; }
    }
    __syncwarp();
    // 2-3. count the entries of every lane's buckets
#pragma unroll
    for (int jj = 0; jj < KPL; ++jj) {
        if (32u * jj >= nk) continue;   // warp-uniform; no break, so the loop unrolls and lo / key stay in registers
        const uint32_t p = lane + 32 * jj;
        const uint32_t sz = lo[jj].y, start = lo[jj].x;
        const uint32_t op0 = p < nk ? s.kpre[p] : 0u;   // dense index of the bucket's first op
        uint32_t q0 = lo[jj].z, q1 = lo[jj].w, q2 = 0, q3 = 0, q4 = 0, q5 = 0;
        if (sz > 2) {
            const uint4 hi = __ldg(ix.rec + 2ull * key[jj] + 1);   // key[jj]: the record's slot
            q2 = hi.x; q3 = hi.y; q4 = hi.z;
            // a hashed slot holds five entries (its last word is the key)
            q5 = !ix.rec_hashed ? hi.w : (sz > 5 ? __ldg(ix.entry + start + 5) : 0u);
        }
        uint32_t jmax = sz;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) jmax = max(jmax, __shfl_xor_sync(FULL, jmax, d));
        uint32_t prev = EMPTY_KEY;
        // sub-step j takes entry j of every lane's bucket; lanes holding the
        // same key add their ops through one leader (same-address atomics from
        // a whole warp would serialise)
        for (uint32_t j = 0; j < jmax; ++j) {
            const uint32_t e = q0;
            q0 = q1; q1 = q2; q2 = q3; q3 = q4; q4 = q5;
            q5 = j + REC_INLINE < sz ? __ldg(ix.entry + start + j + REC_INLINE) : 0u;
            const bool valid = j < sz && !(j > 0 && prev == e);
            prev = e;
            const unsigned vm = __ballot_sync(FULL, valid);
            const unsigned tm = __ballot_sync(FULL, valid && p > maxQPos);
            const unsigned grp = __match_any_sync(FULL, valid ? e : EMPTY_KEY) & vm;
            bool reach = false;
            uint32_t h = 0;
            if (valid && (uint32_t)(__ffs(grp) - 1) == lane) {
                h = dt_hash(e, DT - 1);
                while (true) {
                    const uint32_t cur = s.dt_key[h];
                    if (cur == e) break;
                    if (cur == EMPTY_KEY) {
                        const uint32_t old = atomicCAS(&s.dt_key[h], EMPTY_KEY, e);
                        if (old == EMPTY_KEY || old == e) break;
                    }
                    h = (h + 1) & (DT - 1);
                }
                // the leader holds the group's lowest k-mer, so its op comes first
                const uint32_t v = s.dt_val[h];
                const uint32_t n = (uint32_t)__popc(grp);
                const uint32_t first = min(dtv_first(v), op0 + j);
                s.dt_val[h] = ((v & ((1u << DTV_FIRST_SHIFT) - 1)) + n + (uint32_t)__popc(grp & tm) * DTV_TAIL) |
                              (first << DTV_FIRST_SHIFT);
                reach = dtv_count(v) < QTHRESH && dtv_count(v) + n >= QTHRESH;
            }
            const unsigned rm = __ballot_sync(FULL, reach);
            if (reach) {
                const uint32_t at = nreached + __popc(rm & ((1u << lane) - 1));
                if (at < 32) s.reached[at] = h;
            }
            nreached += __popc(rm);
            __syncwarp();   // this sub-step's count-table writes before the next one's probes
        }
    }
    __syncwarp();
    // 4. both strand maps with at most one candidate (count >= QTHRESH,
    //    inserted): no insertion order needed; staged at once, forward map
    //    first (the order saQuerySeedSetRef walks)
    if (nreached <= 32) {
        uint32_t k = 0;
        bool cand = false;
        if (lane < nreached) {
            const uint32_t h = s.reached[lane];
            cand = dtv_inserted(s.dt_val[h]);
            k = s.dt_key[h];
        }
        const unsigned fm = __ballot_sync(FULL, cand && (k >> 31));
        const unsigned bm = __ballot_sync(FULL, cand && !(k >> 31));
        if (__popc(fm) <= 1 && __popc(bm) <= 1) {
            uint32_t* stg = s.reached + 33;
            const uint32_t nf = __popc(fm), nstage = nf + __popc(bm);
            if (cand) stg[(k >> 31) ? 0 : nf] = k;
            __syncwarp();
            seed_publish(cb, res, task, stg, nstage, nf);
            return 0;
        }
    }
    const int staged = seed_rec_replay<L, OPS, DT, OVF_N>(base, cb.ctr, T);
    if (staged < 0) return 1;
    seed_publish(cb, res, task, s.stage, (uint32_t)staged & 0xffffu, (uint32_t)staged >> 16);
    return 0;
}

// The rest of seed_task_rec when a strand map has two or more candidates
// (about one task in eight at genome scale): the insertion order and the
// replay, kept out of line so that the common path's registers stay its own.
// Returns nstage | nf << 16 with the candidates in s.stage, or -1 when a cap
// is exceeded.
template <class L, uint32_t OPS, uint32_t DT, uint32_t OVF_N>
__device__ __noinline__ int seed_rec_replay(uint8_t* base, unsigned long long* ctr, uint32_t T)
{
    constexpr uint32_t FULL = 0xffffffffu;
    const SeedMemR s = seed_mem_r<L, OPS, DT, OVF_N>(base);
    const uint32_t lane = threadIdx.x & 31;
    if (lane == 0) atomicAdd(ctr + CTR_REPLAY, 1ull);
    // 4b. the inserted keys in first-touch order: each inserted key marks the
    //     dense index of its first op in a bitmap (first ops of distinct keys
    //     are distinct ops); a key's rank is the number of marks below its own
    s.bitmap[lane] = 0;
    __syncwarp();
    for (uint32_t b0 = 0; b0 < DT; b0 += 32) {
        const uint32_t h = b0 + lane;
        if (s.dt_key[h] != EMPTY_KEY) {
            const uint32_t v = s.dt_val[h];
            if (dtv_inserted(v)) {
                const uint32_t d = dtv_first(v);
                atomicOr(&s.bitmap[d >> 5], 1u << (d & 31));
            }
        }
    }
    __syncwarp();
    const uint32_t word = s.bitmap[lane];
    uint32_t wbase = __popc(word);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, wbase, d);
        if (lane >= (uint32_t)d) wbase += t;
    }
    const uint32_t nins = __shfl_sync(FULL, wbase, 31);
    wbase -= __popc(word);
    for (uint32_t b0 = 0; b0 < DT; b0 += 32) {
        const uint32_t h = b0 + lane;
        const uint32_t kk = s.dt_key[h];
        bool take = false;
        uint32_t d = 0, v = 0;
        if (kk != EMPTY_KEY) {
            v = s.dt_val[h];
            take = dtv_inserted(v);
            d = dtv_first(v);
        }
        const uint32_t wb = __shfl_sync(FULL, wbase, take ? (d >> 5) : 0u);
        if (take) {
            const uint32_t rank = wb + __popc(s.bitmap[d >> 5] & ((1u << (d & 31)) - 1));
            s.ins[rank] = kk;
            s.ins_cnt[rank] = (uint16_t)dtv_count(v);
        }
    }
    __syncwarp();
    // 5. replay both maps (forward map first, the order saQuerySeedSetRef
    //    walks); the count table and per-k-mer arrays are dead from here
    SeedMem sm{};
    sm.ins = s.ins;
    sm.slot = s.slot;
    sm.stk = s.stk;
    sm.ovf = s.ovf;
    sm.slot_cap = s.slot_cap;
    sm.stk_cap = s.stk_cap;
    sm.ovf_cap = s.ovf_cap;
    uint32_t nstage = 0, nf = 0;
    for (int dir = 1; dir >= 0; --dir) {
        uint32_t ndc = 0, only = 0;
        for (uint32_t b0 = 0; b0 < nins; b0 += 32) {
            const uint32_t x = b0 + lane;
            const uint32_t v = x < nins ? s.ins[x] : 0u;
            const bool take = x < nins && (v >> 31) == (uint32_t)dir && s.ins_cnt[x] >= QTHRESH;
            const unsigned bm = __ballot_sync(FULL, take);
            if (bm) {
                const uint32_t first = __shfl_sync(FULL, v, __ffs(bm) - 1);
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
        sim_init(m, T / 5);   // bucket_count = summed bucket sizes / 5 (getSeedRefs)
        m.nb = 0; m.novf = 0; m.sp = 0;
        if (m.size > sm.slot_cap) return -1;
        for (uint32_t b = lane; b < m.size; b += 32) sm.slot[b] = EMPTY_KEY;
        __syncwarp();
        for (uint32_t b0 = 0; b0 < nins; b0 += 32) {
            const uint32_t xl = b0 + lane;
            const unsigned todo = __ballot_sync(FULL, xl < nins && (s.ins[xl] >> 31) == (uint32_t)dir);
            if (!sim_insert_batch_w(m, sm, b0, todo)) return -1;
        }
        __syncwarp();
        // iteration order: buckets in array order, then the overflow list
        for (uint32_t b0 = 0; b0 < m.size + m.novf; b0 += 32) {
            const uint32_t b = b0 + lane;
            uint32_t x = EMPTY_KEY;
            if (b < m.size) x = sm.slot[b];
            else if (b < m.size + m.novf) x = sm.ovf[b - m.size];
            const bool take = x != EMPTY_KEY && s.ins_cnt[x] >= QTHRESH;
            const unsigned bm = __ballot_sync(FULL, take);
            if (take) s.stage[nstage + __popc(bm & ((1u << lane) - 1))] = s.ins[x];
            nstage += __popc(bm);
        }
        __syncwarp();
        if (dir == 1) nf = nstage;
    }
    return (int)(nstage | nf << 16);
}

}  // namespace fame
