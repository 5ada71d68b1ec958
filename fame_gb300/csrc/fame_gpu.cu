// C ABI implementation: index upload, per-chunk matching pipeline, tallies.
#include <cuda_runtime.h>

#include <sys/mman.h>
#include <sys/syscall.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fame_gpu.h"
#include "index_host.h"
#include "internal.h"
#include "pe.cuh"

using namespace fame;

struct fame_gpu {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex host_mu;
    std::unordered_map<void*, size_t> host_mapped;   // page-locked blocks placed by host_alloc_near
    std::string err;
    DevIndex ix{};
    std::vector<void*> index_allocs;
    uint64_t index_bytes = 0;            // device bytes of the resident index tables
    int rec_layout = FAME_REC_DENSE;     // bucket-record layout (FAME_REC_DENSE / FAME_REC_HASHED)
    uint64_t rec_slots = 0;              // records (dense: HTABSIZE; hashed: slots of the table)
    uint64_t nonempty_buckets = 0;
    uint64_t n_cpg = 0;
    uint32_t max_bucket = 0;
    // chunk buffers
    uint64_t cap_reads = 0, cap_bytes = 0, cap_cand = 0;
    char* d_seqs = nullptr;
    uint64_t* d_offs = nullptr;
    uint8_t* d_rflags = nullptr;
    uint4* d_task_cand = nullptr;
    uint32_t *d_cand = nullptr, *d_cand_task = nullptr, *d_hits = nullptr, *d_hit_n = nullptr;
    uint8_t* d_cand_flags = nullptr;
    uint64_t* d_mats = nullptr;
    uint8_t* d_invalid = nullptr;
    uint32_t* d_dp_list = nullptr;
    uint64_t* d_dp_mat = nullptr;
    uint8_t* d_dp_orient = nullptr;
    uint32_t* d_heavy = nullptr;
    uint32_t* d_heavy2 = nullptr;
    unsigned long long* d_ctr = nullptr;
    unsigned long long* h_ctr = nullptr;  // pinned
    uint32_t* d_meth = nullptr;
    uint16_t* d_meth16 = nullptr;        // packed tallies on their way to the host (allocated at first read)
    HeavyScratch hs{};                   // large-capacity seeding tier (caps from the largest bucket)
    HeavyScratch ms{};                   // global-memory middle seeding tier (genome-scale buckets, many warps)
    int seed_mid_first = 0;              // 1: every task seeds in the middle tiers (k_seed_route), no light attempt
    int mid_skip_small = 0;              // 1: the middle tiers start at the larger one
    uint32_t mid_grid[2] = {0, 0};       // resident blocks of the smaller and the larger middle tier
    int timing = 0;
    cudaEvent_t ev[12]{};
    float stage_ms[FAME_STAGES]{};
    float pe_stage_ms[FAME_PAIR_STAGES]{};
    uint64_t tier_tasks[5]{};            // tasks entering each seeding tier after the light one, last chunk;
                                         // [4]: tasks whose candidate order needed the map replay
    int launches = 0;
    int sm_count = 0;
    uint32_t dp_grid = 0;   // resident blocks of k_dp_warp on the whole device
    uint32_t dp_blocks = 0; // blocks k_dp_warp is launched with (the autotuner may pick fewer)
    uint32_t sa_blocks_per_sm = 32;      // k_shiftand blocks per SM (its warps loop over the candidates)
    // paired path
    PeIndex px{};
    uint64_t pe_warp_bytes = 0;          // shared memory per warp of k_pe_seed
    uint32_t pe_grid = 0;                // resident blocks of k_pe_seed
    PeTaskRec* d_pe_recs = nullptr;      // per pair orientation
    uint64_t cap_pe_recs = 0;
    uint8_t* d_pe_heavy = nullptr;       // global scratch of k_pe_heavy
    uint8_t* d_pe_mid = nullptr;         // global scratch of the paired middle tiers (PE_MID_S, then PE_MID)
    uint8_t* d_pe_mid2 = nullptr;
    uint64_t pe_mid_warp_bytes = 0, pe_mid2_warp_bytes = 0;
    uint32_t pe_mid_warps = 0, pe_mid2_warps = 0;
    uint64_t pe_heavy_warp_bytes = 0;
    uint32_t pe_heavy_warps = 0;
    fame_queue* queue = nullptr;         // the batched form's slots, if open
    uint8_t* noalloc_scratch = nullptr;  // device address of the no-allocation entry point's static array
};

void queue_quiesce(fame_queue* q);
// Waits for the queue's slots and drops their captured graphs (launch shapes
// changed; the next chunk of each shape is captured again).
void queue_drop_graphs(fame_queue* q);
// Device address of the static scratch array of fame_gpu_call_cpgs_noalloc on
// the current device (defined with the array, below).
cudaError_t noalloc_scratch_address(void** p);

namespace {

int set_err(fame_gpu* g, int code, const std::string& msg)
{
    if (g) g->err = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return set_err(g, e_ == cudaErrorMemoryAllocation ? FAME_ERR_NOMEM : FAME_ERR_CUDA,    \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

template <class T>
int dev_alloc(fame_gpu* g, T** p, uint64_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc((void**)p, count * sizeof(T)));
    return FAME_OK;
}

template <class T>
void dev_free(T*& p)
{
    if (p) cudaFree((void*)p);
    p = nullptr;
}

// Bucket entries a read's k-mers may gather in the middle seeding tier.
constexpr uint32_t MID_OPS = 4096;

// Heavy-pair caps: keys per map and phase, value-table slots, replayed buckets
// (bucket_count = summed bucket sizes / 5 <= 224 k-mers x KMERCUTOFF / 5).
constexpr PeCaps PE_HEAVY{16384, 65536, 131072 + NBHD - 1 + 64, 4096, 4096, 0, PE_KMAX};

// Page-locked host memory on the host NUMA node nearest the device (anonymous
// pages bound there with mbind, touched, then registered with CUDA), so
// host-device copies do not cross to another socket's memory; cudaMallocHost
// when the node is unknown or the placement is refused.
void* host_alloc_near(fame_gpu* g, size_t bytes)
{
    bytes = std::max<size_t>(bytes, 16);
    int node = -1;
    if (cudaDeviceGetAttribute(&node, cudaDevAttrHostNumaId, g->device) != cudaSuccess) node = -1;
    if (node >= 0 && node < 64) {
        const size_t pg = (size_t)sysconf(_SC_PAGESIZE);
        const size_t len = (bytes + pg - 1) / pg * pg;
        void* m = mmap(nullptr, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
        if (m != MAP_FAILED) {
            unsigned long mask = 1ul << node;
            const long MPOL_PREFERRED_ = 1;
            if (syscall(SYS_mbind, m, len, MPOL_PREFERRED_, &mask, 65ul, 0u) == 0) {
                // huge pages where the host has them: far fewer pages to pin and to map
                // for the device's copies (the first copy from a buffer of 4 KiB or
                // 64 KiB pages was measured at half the rate of later ones)
                madvise(m, len, MADV_HUGEPAGE);
                std::memset(m, 0, len);
                if (cudaHostRegister(m, len, cudaHostRegisterDefault) == cudaSuccess) {
                    std::lock_guard<std::mutex> lk(g->host_mu);
                    g->host_mapped[m] = len;
                    return m;
                }
                cudaGetLastError();
            }
            munmap(m, len);
        }
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}

void host_free_near(fame_gpu* g, void* p)
{
    if (!p) return;
    size_t len = 0;
    {
        std::lock_guard<std::mutex> lk(g->host_mu);
        auto it = g->host_mapped.find(p);
        if (it != g->host_mapped.end()) {
            len = it->second;
            g->host_mapped.erase(it);
        }
    }
    if (len) {
        cudaHostUnregister(p);
        munmap(p, len);
    } else {
        cudaFreeHost(p);
    }
}

int grow_chunk(fame_gpu* g, uint64_t n, uint64_t bytes, uint64_t cand)
{
    int rc;
    if (n > g->cap_reads) {
        const uint64_t c = std::max<uint64_t>(n, 1024);
        dev_free(g->d_offs); dev_free(g->d_rflags); dev_free(g->d_task_cand); dev_free(g->d_mats);
        dev_free(g->d_invalid); dev_free(g->d_dp_list); dev_free(g->d_dp_mat); dev_free(g->d_dp_orient);
        dev_free(g->d_heavy); dev_free(g->d_heavy2);
        if ((rc = dev_alloc(g, &g->d_offs, c + 1)) || (rc = dev_alloc(g, &g->d_rflags, c)) ||
            (rc = dev_alloc(g, &g->d_task_cand, 2 * c)) || (rc = dev_alloc(g, &g->d_mats, c)) ||
            (rc = dev_alloc(g, &g->d_invalid, c)) || (rc = dev_alloc(g, &g->d_dp_list, c)) ||
            (rc = dev_alloc(g, &g->d_dp_mat, c)) || (rc = dev_alloc(g, &g->d_dp_orient, c)) ||
            (rc = dev_alloc(g, &g->d_heavy, 2 * c)) || (rc = dev_alloc(g, &g->d_heavy2, 2 * c)))
            return rc;
        g->cap_reads = c;
    }
    if (bytes > g->cap_bytes) {
        const uint64_t c = std::max<uint64_t>(bytes, 1 << 20);
        dev_free(g->d_seqs);
        if ((rc = dev_alloc(g, &g->d_seqs, c))) return rc;
        g->cap_bytes = c;
    }
    if (cand > g->cap_cand) {
        const uint64_t c = std::max<uint64_t>(cand, 1 << 16);
        dev_free(g->d_cand); dev_free(g->d_cand_task); dev_free(g->d_hits); dev_free(g->d_hit_n);
        dev_free(g->d_cand_flags);
        if ((rc = dev_alloc(g, &g->d_cand, c)) || (rc = dev_alloc(g, &g->d_cand_task, c)) ||
            (rc = dev_alloc(g, &g->d_hits, c * HIT_CAP)) || (rc = dev_alloc(g, &g->d_hit_n, c)) ||
            (rc = dev_alloc(g, &g->d_cand_flags, c)))
            return rc;
        g->cap_cand = c;
    }
    return FAME_OK;
}

// fn(begin, end) over up to 16 host threads (the index upload's staging
// loops, which are per-element and independent).  fn must not throw.
template <class F>
void host_par(uint64_t n, F fn)
{
    const int T = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (T <= 1 || n < (1u << 16)) { fn(0, n); return; }
    std::vector<std::thread> th;
    const uint64_t step = (n + T - 1) / T;
    for (int t = 0; t < T; ++t) {
        const uint64_t b = std::min<uint64_t>(n, (uint64_t)t * step), e = std::min<uint64_t>(n, b + step);
        if (b >= e) break;
        try {
            th.emplace_back([=] { fn(b, e); });
        } catch (...) {
            fn(b, e);
        }
    }
    for (auto& x : th) x.join();
}

uint32_t pow2_ceil_host(uint64_t v)
{
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return (uint32_t)p;
}

}  // namespace

extern "C" const char* fame_gpu_last_error(const fame_gpu* g) { return g ? g->err.c_str() : "null context"; }

int fame_gpu_fail(fame_gpu* g, int code, const char* msg) { return set_err(g, code, msg ? msg : ""); }
int fame_gpu_device_of(const fame_gpu* g) { return g ? g->device : -1; }

extern "C" int fame_gpu_close(fame_gpu* g)
{
    if (!g) return FAME_ERR_ARG;
    cudaSetDevice(g->device);
    if (g->queue) fame_queue_close(g->queue);
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (void* p : g->index_allocs) cudaFree(p);
    dev_free(g->d_seqs); dev_free(g->d_offs); dev_free(g->d_rflags); dev_free(g->d_task_cand);
    dev_free(g->d_cand); dev_free(g->d_cand_task); dev_free(g->d_hits); dev_free(g->d_hit_n);
    dev_free(g->d_mats); dev_free(g->d_invalid); dev_free(g->d_dp_list); dev_free(g->d_dp_mat);
    dev_free(g->d_dp_orient); dev_free(g->d_heavy); dev_free(g->d_heavy2); dev_free(g->d_ctr); dev_free(g->d_meth);
    dev_free(g->hs.base);
    dev_free(g->ms.base);
    dev_free(g->d_pe_mid);
    dev_free(g->d_pe_mid2);
    dev_free(g->d_meth16);
    dev_free(g->d_pe_heavy);
    dev_free(g->d_pe_recs);
    dev_free(g->d_cand_flags);
    if (g->h_ctr) cudaFreeHost(g->h_ctr);
    for (auto& e : g->ev) if (e) cudaEventDestroy(e);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return FAME_OK;
}

extern "C" int fame_gpu_open(const fame_index_view* v, int device, fame_gpu** out)
{
    return fame_gpu_open_layout(v, device, FAME_REC_AUTO, out);
}

extern "C" int fame_gpu_open_layout(const fame_index_view* v, int device, int layout, fame_gpu** out)
{
    if (!v || !out || layout < FAME_REC_AUTO || layout > FAME_REC_HASHED) return FAME_ERR_ARG;
    *out = nullptr;
    fame_gpu* g = new (std::nothrow) fame_gpu();
    if (!g) return FAME_ERR_NOMEM;
    auto fail = [&](int rc) { *out = nullptr; std::string m = g->err; fame_gpu_close(g); (void)m; return rc; };
    g->device = device;
    if (cudaSetDevice(device) != cudaSuccess) return fail(set_err(g, FAME_ERR_CUDA, "cudaSetDevice failed"));
    cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(set_err(g, FAME_ERR_CUDA, "cudaStreamCreate failed"));
    for (auto& e : g->ev) cudaEventCreate(&e);
    // ---- validate the view
    if (v->n_chrom == 0 || v->n_chrom > 256 || !v->chrom_seq || !v->chrom_len || !v->kmer ||
        (!v->tab_index && !v->tab_index32) || (!v->strand_bits && v->n_kmer) || !v->win ||
        (!v->cpg && v->n_cpg) || v->readlen <= KMERLEN || v->readlen >= WINLEN)
        return fail(set_err(g, FAME_ERR_INDEX, "incomplete index view"));
    if (v->n_kmer >= 0xffffffffull || v->n_win >= 0x7fffffffull || v->n_cpg >= 0xffffffffull)
        return fail(set_err(g, FAME_ERR_INDEX, "index tables exceed 32-bit device offsets"));
    g->ix.readlen = v->readlen;
    g->ix.n_chrom = v->n_chrom;
    g->ix.n_cpg = v->n_cpg;
    g->ix.n_win = v->n_win;
    g->n_cpg = v->n_cpg;
    auto alloc_idx = [&](void** p, uint64_t bytes) -> int {
        if (cudaMalloc(p, std::max<uint64_t>(bytes, 16)) != cudaSuccess)
            return set_err(g, FAME_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed");
        g->index_allocs.push_back(*p);
        g->index_bytes += bytes;
        return FAME_OK;
    };
    int rc;
    // ---- tabIndex -> uint32 offsets
    uint32_t* d_tab;
    if ((rc = alloc_idx((void**)&d_tab, (HTABSIZE + 1) * 4))) return fail(rc);
    const uint64_t CH = 1ull << 26;
    std::vector<uint32_t> stage(CH);
    if (v->tab_index32) {
        if (v->tab_index32[HTABSIZE] != v->n_kmer) return fail(set_err(g, FAME_ERR_INDEX, "tabIndex end != k-mer count"));
        if (cudaMemcpy(d_tab, v->tab_index32, (HTABSIZE + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_CUDA, "tabIndex upload failed"));
    } else {
        if (v->tab_index[HTABSIZE] != v->n_kmer) return fail(set_err(g, FAME_ERR_INDEX, "tabIndex end != k-mer count"));
        for (uint64_t b = 0; b < HTABSIZE + 1; b += CH) {
            const uint64_t e = std::min<uint64_t>(HTABSIZE + 1, b + CH);
            host_par(e - b, [&](uint64_t i0, uint64_t i1) {
                for (uint64_t i = i0; i < i1; ++i) stage[i] = (uint32_t)v->tab_index[b + i];
            });
            if (cudaMemcpy(d_tab + b, stage.data(), (e - b) * 4, cudaMemcpyHostToDevice) != cudaSuccess)
                return fail(set_err(g, FAME_ERR_CUDA, "tabIndex upload failed"));
        }
    }

    // ---- entries: window id | forward << 31
    uint32_t* d_entry;
    if ((rc = alloc_idx((void**)&d_entry, v->n_kmer * 4))) return fail(rc);
    for (uint64_t b = 0; b < v->n_kmer; b += CH) {
        const uint64_t e = std::min<uint64_t>(v->n_kmer, b + CH);
        std::atomic<uint64_t> bad{~0ull};
        host_par(e - b, [&](uint64_t i0, uint64_t i1) {
            for (uint64_t j = i0; j < i1; ++j) {
                const uint64_t i = b + j;
                const uint32_t meta = v->kmer[i].meta;
                if ((meta >> 31) || meta >= v->n_win) {
                    uint64_t cur = bad.load();
                    while (i < cur && !bad.compare_exchange_weak(cur, i)) {}
                }
                const uint32_t fwd = (v->strand_bits[i >> 3] >> (i & 7)) & 1u;
                stage[j] = meta | (fwd << 31);
            }
        });
        if (bad.load() != ~0ull)
            return fail(set_err(g, FAME_ERR_INDEX, "k-mer entry " + std::to_string(bad.load()) + " has a start-CpG flag or an unknown window"));
        if (cudaMemcpy(d_entry + b, stage.data(), (e - b) * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_CUDA, "k-mer upload failed"));
    }
    g->ix.entry = d_entry;
    // ---- bucket records: start, size and the first entries of each bucket in one sector;
    //      dense (one record per bucket) or hashed (the non-empty buckets only)
    {
        unsigned long long* d_cnt;
        if (cudaMalloc((void**)&d_cnt, 8) != cudaSuccess) return fail(set_err(g, FAME_ERR_NOMEM, "alloc"));
        unsigned long long nne = 0;
        cudaMemsetAsync(d_cnt, 0, 8, g->stream);
        k_count_nonempty<<<g->sm_count * 8, 256, 0, g->stream>>>(d_tab, HTABSIZE, d_cnt);
        cudaMemcpyAsync(&nne, d_cnt, 8, cudaMemcpyDeviceToHost, g->stream);
        const cudaError_t ce = cudaStreamSynchronize(g->stream);
        cudaFree(d_cnt);
        if (ce != cudaSuccess) return fail(set_err(g, FAME_ERR_CUDA, "bucket count failed"));
        g->nonempty_buckets = nne;
        uint64_t slots = 1024;
        while (slots < 2 * nne) slots <<= 1;
        const bool hashed = layout == FAME_REC_HASHED || (layout == FAME_REC_AUTO && 4 * nne <= HTABSIZE);
        if (hashed && slots > HTABSIZE)
            return fail(set_err(g, FAME_ERR_INDEX, "hashed bucket records need at most HTABSIZE / 2 non-empty buckets"));
        uint4* d_rec;
        if (hashed) {
            if ((rc = alloc_idx((void**)&d_rec, slots * 32))) return fail(rc);
            cudaMemsetAsync(d_rec, 0xff, slots * 32, g->stream);
            k_build_rec_hashed<<<g->sm_count * 8, 256, 0, g->stream>>>(d_tab, d_entry, HTABSIZE, d_rec,
                                                                        (uint32_t)(slots - 1));
            g->ix.rec_mask = (uint32_t)(slots - 1);
            g->ix.rec_hashed = 1;
            g->rec_layout = FAME_REC_HASHED;
            g->rec_slots = slots;
        } else {
            if ((rc = alloc_idx((void**)&d_rec, HTABSIZE * 32))) return fail(rc);
            k_build_rec<<<g->sm_count * 8, 256, 0, g->stream>>>(d_tab, d_entry, HTABSIZE, d_rec);
            g->ix.rec_mask = (uint32_t)HTAB_MASK;
            g->ix.rec_hashed = 0;
            g->rec_layout = FAME_REC_DENSE;
            g->rec_slots = HTABSIZE;
        }
        if (cudaGetLastError() != cudaSuccess) return fail(set_err(g, FAME_ERR_CUDA, "bucket record build failed"));
        g->ix.rec = d_rec;
    }
    // ---- paired path: tmask per entry (kmerTableSmall.tmask), filteredKmers sorted
    {
        uint32_t* d_tm;
        if ((rc = alloc_idx((void**)&d_tm, v->n_kmer * 4))) return fail(rc);
        for (uint64_t b = 0; b < v->n_kmer; b += CH) {
            const uint64_t e = std::min<uint64_t>(v->n_kmer, b + CH);
            host_par(e - b, [&](uint64_t i0, uint64_t i1) {
                for (uint64_t i = i0; i < i1; ++i) stage[i] = v->kmer[b + i].tmask;
            });
            if (cudaMemcpy(d_tm + b, stage.data(), (e - b) * 4, cudaMemcpyHostToDevice) != cudaSuccess)
                return fail(set_err(g, FAME_ERR_CUDA, "tmask upload failed"));
        }
        std::vector<uint64_t> f;
        if (v->n_filtered && v->filtered) f.assign(v->filtered, v->filtered + v->n_filtered);
        std::sort(f.begin(), f.end());
        uint64_t* d_f;
        if ((rc = alloc_idx((void**)&d_f, f.size() * 8))) return fail(rc);
        if (!f.empty() && cudaMemcpy(d_f, f.data(), f.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_CUDA, "filteredKmers upload failed"));
        g->px.tmask = d_tm;
        g->px.filtered = d_f;
        g->px.n_filtered = f.size();
    }
    // ---- genome: 2-bit codes + N mask, chromosomes at 32-base aligned offsets
    std::vector<uint64_t> coff(v->n_chrom), clen(v->n_chrom);
    uint64_t tot = 0;
    for (uint32_t c = 0; c < v->n_chrom; ++c) { coff[c] = tot; clen[c] = v->chrom_len[c]; tot += (clen[c] + 31) / 32 * 32; }
    {
        // 32 bases per step: two packed words and one N-mask word, so threads
        // never share a word (chromosomes start at 32-base boundaries)
        std::vector<uint32_t> pack(tot / 16 + 1, 0), nm(tot / 32 + 1, 0);
        for (uint32_t c = 0; c < v->n_chrom; ++c) {
            const char* s = v->chrom_seq[c];
            const uint64_t L = clen[c];
            std::atomic<int> bad{0};
            host_par((L + 31) / 32, [&](uint64_t q0, uint64_t q1) {
                for (uint64_t q = q0; q < q1; ++q) {
                    uint32_t w0 = 0, w1 = 0, nmask = 0;
                    const uint64_t i0 = 32 * q, i1 = std::min<uint64_t>(L, i0 + 32);
                    for (uint64_t i = i0; i < i1; ++i) {
                        const uint32_t k = (uint32_t)(i - i0);
                        uint32_t code = 0;
                        switch (s[i]) {
                            case 'A': code = 0; break;
                            case 'C': code = 1; break;
                            case 'G': code = 2; break;
                            case 'T': code = 3; break;
                            case 'N': nmask |= 1u << k; break;
                            default: bad = 1; break;
                        }
                        if (k < 16) w0 |= code << (2 * k);
                        else w1 |= code << (2 * (k - 16));
                    }
                    const uint64_t gi = coff[c] + i0;
                    pack[gi >> 4] = w0;
                    pack[(gi >> 4) + 1] = w1;
                    nm[gi >> 5] = nmask;
                }
            });
            if (bad.load())
                return fail(set_err(g, FAME_ERR_INDEX, "reference base outside ACGTN in chromosome " + std::to_string(c)));
        }
        uint32_t *d_pack, *d_nm;
        uint64_t *d_coff, *d_clen;
        if ((rc = alloc_idx((void**)&d_pack, pack.size() * 4)) || (rc = alloc_idx((void**)&d_nm, nm.size() * 4)) ||
            (rc = alloc_idx((void**)&d_coff, coff.size() * 8)) || (rc = alloc_idx((void**)&d_clen, clen.size() * 8)))
            return fail(rc);
        if (cudaMemcpy(d_pack, pack.data(), pack.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d_nm, nm.data(), nm.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d_coff, coff.data(), coff.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d_clen, clen.data(), clen.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_CUDA, "genome upload failed"));
        g->ix.gpack = d_pack; g->ix.gnmask = d_nm; g->ix.chrom_off = d_coff; g->ix.chrom_len = d_clen;
    }
    // ---- windows and CpGs
    {
        std::vector<uint4> w(v->n_win);
        for (uint64_t i = 0; i < v->n_win; ++i) {
            if (v->win[i].chrom >= v->n_chrom) return fail(set_err(g, FAME_ERR_INDEX, "window on unknown chromosome"));
            if (v->win[i].start_ind != CPGDUMMY && (v->win[i].start_ind >= v->n_cpg || (v->win[i].end_ind != CPGDUMMY && v->win[i].end_ind >= v->n_cpg)))
                return fail(set_err(g, FAME_ERR_INDEX, "window CpG range outside cpgTable"));
            w[i] = make_uint4(v->win[i].start_pos, v->win[i].chrom, v->win[i].start_ind, v->win[i].end_ind);
        }
        std::vector<uint32_t> pos(v->n_cpg);
        std::vector<uint8_t> chr(v->n_cpg);
        for (uint64_t i = 0; i < v->n_cpg; ++i) { pos[i] = v->cpg[i].pos; chr[i] = v->cpg[i].chrom; }
        uint4* d_win;
        uint32_t* d_pos;
        uint8_t* d_chr;
        if ((rc = alloc_idx((void**)&d_win, w.size() * 16)) || (rc = alloc_idx((void**)&d_pos, pos.size() * 4)) ||
            (rc = alloc_idx((void**)&d_chr, chr.size())))
            return fail(rc);
        if (cudaMemcpy(d_win, w.data(), w.size() * 16, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d_pos, pos.data(), pos.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d_chr, chr.data(), chr.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_CUDA, "window/CpG upload failed"));
        g->ix.win = d_win; g->ix.cpg_pos = d_pos; g->ix.cpg_chrom = d_chr;
    }
    // ---- largest bucket -> heavy-path scratch
    {
        unsigned int* d_mx;
        if (cudaMalloc(&d_mx, 4) != cudaSuccess) return fail(set_err(g, FAME_ERR_NOMEM, "alloc"));
        cudaMemset(d_mx, 0, 4);
        k_max_bucket<<<g->sm_count * 8, 256, 0, g->stream>>>(d_tab, HTABSIZE, d_mx);
        unsigned int mx = 0;
        cudaMemcpyAsync(&mx, d_mx, 4, cudaMemcpyDeviceToHost, g->stream);
        cudaStreamSynchronize(g->stream);
        // the plain offset table is not needed any more (the records hold the offsets)
        cudaFree(d_tab);
        g->index_bytes -= (HTABSIZE + 1) * 4;
        g->index_allocs.erase(std::remove(g->index_allocs.begin(), g->index_allocs.end(), (void*)d_tab),
                              g->index_allocs.end());
        if (cudaStreamSynchronize(g->stream) != cudaSuccess) { cudaFree(d_mx); return fail(set_err(g, FAME_ERR_CUDA, "bucket scan failed")); }
        cudaFree(d_mx);
        g->max_bucket = mx;
        const uint64_t ops_cap = std::max<uint64_t>(L_OPS + 1, std::min<uint64_t>((uint64_t)224 * std::max(1u, mx), 1ull << 24));
        g->hs.ops_cap = (uint32_t)ops_cap;
        g->hs.dt_cap = pow2_ceil_host(2 * ops_cap + 2);
        g->hs.slot_cap = 2 * pow2_ceil_host(ops_cap + 1) + 64;
        g->hs.bytes_per_warp = heavy_bytes_per_warp(g->hs.ops_cap, g->hs.dt_cap, g->hs.slot_cap);
        g->hs.nwarps = (uint32_t)std::max<uint64_t>(8, std::min<uint64_t>(256, (4ull << 30) / g->hs.bytes_per_warp));
        if (cudaMalloc(&g->hs.base, g->hs.bytes_per_warp * g->hs.nwarps) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_NOMEM, "heavy-path scratch allocation failed"));
        // middle tier: reads whose k-mers gather up to MID_OPS bucket entries
        // (genome-scale indexes hold about three entries per bucket, so most
        // reads exceed the shared-memory caps), 16 warps per SM
        g->ms.ops_cap = MID_OPS;
        g->ms.dt_cap = pow2_ceil_host(2 * MID_OPS + 2);
        g->ms.slot_cap = 2 * pow2_ceil_host(MID_OPS + 1) + 64;
        g->ms.bytes_per_warp = heavy_bytes_per_warp(g->ms.ops_cap, g->ms.dt_cap, g->ms.slot_cap);
        g->ms.nwarps = (uint32_t)g->sm_count * 16;
        // with more than one entry per bucket on average (genome-scale
        // indexes) nearly every read exceeds the shared-memory caps
        g->seed_mid_first = v->n_kmer > HTABSIZE ? 1 : 0;
        if (cudaMalloc(&g->ms.base, g->ms.bytes_per_warp * g->ms.nwarps) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_NOMEM, "middle-tier seeding scratch allocation failed"));
        // shared-memory middle tiers: resident blocks per SM from their
        // shared-memory footprints
        const void* fns[2] = {(const void*)k_seed_mid<MID_S_OPS, MID_S_DT, MID_S_WPB>,
                              (const void*)k_seed_mid<MID_L_OPS, MID_L_DT, MID_L_WPB>};
        const uint32_t sbytes[2] = {MID_S_WPB * MidS::BYTES, MID_L_WPB * MidL::BYTES};
        const int threads[2] = {32 * MID_S_WPB, 32 * MID_L_WPB};
        for (int k = 0; k < 2; ++k) {
            int nb = 0;
            if (cudaFuncSetAttribute(fns[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sbytes[k]) != cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fns[k], threads[k], sbytes[k]) != cudaSuccess || nb < 1)
                return fail(set_err(g, FAME_ERR_CUDA, "k_seed_mid does not fit an SM"));
            g->mid_grid[k] = (uint32_t)(g->sm_count * nb);
        }
    }
    // ---- tallies, counters, DP scratch
    if ((rc = dev_alloc(g, &g->d_meth, 4 * std::max<uint64_t>(1, v->n_cpg)))) return fail(rc);
    if (cudaMemset(g->d_meth, 0, 16 * std::max<uint64_t>(1, v->n_cpg)) != cudaSuccess) return fail(set_err(g, FAME_ERR_CUDA, "memset"));
    if ((rc = dev_alloc(g, &g->d_ctr, CTR_N))) return fail(rc);
    if (cudaMallocHost(&g->h_ctr, CTR_N * sizeof(unsigned long long)) != cudaSuccess) return fail(set_err(g, FAME_ERR_NOMEM, "pinned alloc"));
    {
        // resolved here, with the device current, so that it follows this
        // context's lifetime (a module reloaded after a device reset may place
        // the array elsewhere) and is known before any stream capture
        void* p = nullptr;
        const cudaError_t e = noalloc_scratch_address(&p);
        if (e != cudaSuccess || !p)
            return fail(set_err(g, FAME_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)));
        g->noalloc_scratch = (uint8_t*)p;
    }
    if (cudaFuncSetAttribute(k_seed, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * LightR::BYTES) != cudaSuccess ||
        cudaFuncSetAttribute(k_dp_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * DPW_BYTES) != cudaSuccess)
        return fail(set_err(g, FAME_ERR_CUDA, "shared memory attribute"));
    {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_dp_warp, 128, 4 * DPW_BYTES) != cudaSuccess || nb < 1)
            return fail(set_err(g, FAME_ERR_CUDA, "k_dp_warp does not fit an SM"));
        g->dp_grid = (uint32_t)(g->sm_count * nb);
        g->dp_blocks = g->dp_grid;
        uint64_t off[PE_LAYOUT_N], hoff[PE_LAYOUT_N], moff[PE_LAYOUT_N], m2off[PE_LAYOUT_N];
        g->pe_warp_bytes = pe_layout(PE_LIGHT, off);
        pe_layout(PE_HEAVY, hoff);
        g->pe_mid_warp_bytes = pe_layout(PE_MID_S, moff);
        g->pe_mid2_warp_bytes = pe_layout(PE_MID, m2off);
        // pe_kmers keeps its per-read arrays (8 * 256 + 96 bytes) in layout regions 11 .. 16
        if (off[17] - off[11] < PE_KMER_AREA || hoff[17] - hoff[11] < PE_KMER_AREA ||
            moff[17] - moff[11] < PE_KMER_AREA || m2off[17] - m2off[11] < PE_KMER_AREA)
            return fail(set_err(g, FAME_ERR_CUDA, "paired layout: k-mer area too small"));
        const size_t pe_smem = PE_SEED_WARPS * g->pe_warp_bytes;   // the largest layout (mates up to 255 bases)
        if (cudaFuncSetAttribute(k_pe_seed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pe_smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pe_seed, 32 * PE_SEED_WARPS, pe_smem) != cudaSuccess || nb < 1)
            return fail(set_err(g, FAME_ERR_CUDA, "k_pe_seed does not fit an SM"));
        g->pe_grid = (uint32_t)(g->sm_count * nb);
    }
    *out = g;
    return FAME_OK;
}

namespace {

// The seeding tiers after the light one (or k_seed_route), every count read
// on the device: the shared-memory middle tiers (unless skipped, the smaller
// first), then the global-memory tier and the large-capacity one, each over
// the tasks the tier before could not hold.  The task lists alternate
// between cb.heavy and cb.heavy2 (a list is fully taken before the next tier
// writes over it).  ev, when given, receives an event after each middle tier
// and after the global-memory tier.  Returns the launches.
int seed_tiers(fame_gpu* g, const ChunkBufs& cb, cudaStream_t st, const HeavyScratch& ms, const HeavyScratch& hs,
               cudaEvent_t* ev = nullptr)
{
    uint32_t* lists[2] = {cb.heavy, cb.heavy2};
    int cur = 0, ctr = CTR_HEAVY, launches = 0;
    const int spill_ctr[3] = {CTR_HEAVY2, CTR_HEAVY3, CTR_HEAVY4};
    int k = 0;
    if (!g->mid_skip_small) {
        k_seed_mid<MID_S_OPS, MID_S_DT, MID_S_WPB><<<g->mid_grid[0], 32 * MID_S_WPB, MID_S_WPB * MidS::BYTES, st>>>(
            g->ix, cb, lists[cur], ctr, CTR_QMID, lists[cur ^ 1], spill_ctr[k]);
        cur ^= 1; ctr = spill_ctr[k++]; ++launches;
    }
    if (ev) cudaEventRecord(ev[0], st);
    k_seed_mid<MID_L_OPS, MID_L_DT, MID_L_WPB><<<g->mid_grid[1], 32 * MID_L_WPB, MID_L_WPB * MidL::BYTES, st>>>(
        g->ix, cb, lists[cur], ctr, CTR_QMID2, lists[cur ^ 1], spill_ctr[k]);
    cur ^= 1; ctr = spill_ctr[k++]; ++launches;
    if (ev) cudaEventRecord(ev[1], st);
    k_seed_tier<<<(ms.nwarps + 3) / 4, 128, 0, st>>>(g->ix, cb, ms, FROM_DEVICE, lists[cur], ctr, lists[cur ^ 1],
                                                     spill_ctr[k]);
    cur ^= 1; ctr = spill_ctr[k]; ++launches;
    if (ev) cudaEventRecord(ev[2], st);
    k_seed_tier<<<(hs.nwarps + 3) / 4, 128, 0, st>>>(g->ix, cb, hs, FROM_DEVICE, lists[cur], ctr, nullptr, 0);
    return launches + 1;
}

int run_chunk(fame_gpu* g, const char* d_seqs, const uint64_t* d_offs, uint32_t n, uint32_t flags, uint64_t* d_mats,
              uint8_t* d_invalid, fame_counters* cnt, uint32_t* meth = nullptr)
{
    const bool both = flags & FAME_BOTH_STRANDS, stranded = flags & FAME_GET_STRANDED;
    const uint32_t omask = (both || stranded) ? 3u : ((flags & FAME_MATCH_R1_FWD) ? 1u : 2u);
    const uint32_t norient = omask == 3u ? 2u : 1u;
    int rc;
    if ((rc = grow_chunk(g, n, 0, (uint64_t)n * norient * 4 + 4096))) return rc;
    ChunkBufs cb{};
    cb.seqs = d_seqs;
    cb.offs = d_offs;
    cb.n = n;
    cb.orient_mask = omask;
    cb.stranded = stranded ? 1u : 0u;
    cb.rflags = g->d_rflags;
    cb.task_cand = g->d_task_cand;
    cb.mats = d_mats;
    cb.invalid = d_invalid;
    cb.dp_list = g->d_dp_list;
    cb.dp_mat = g->d_dp_mat;
    cb.dp_orient = g->d_dp_orient;
    cb.meth = meth ? meth : g->d_meth;
    cb.ctr = g->d_ctr;
    cb.heavy = g->d_heavy;
    cb.heavy2 = g->d_heavy2;
    const int T = g->timing;
    g->launches = 0;
    if (g->queue) queue_quiesce(g->queue);   // the queue's slots share the heavy-path scratch
    // The whole chunk is enqueued at once, every count read on the device
    // (FROM_DEVICE): the heavy-read seeding and the automaton widths without
    // work return at once, and the later stages stop when the candidate buffer
    // overflowed, in which case nothing was tallied and the chunk runs again
    // with a larger buffer.  One host wait per pass.
    for (int attempt = 0; attempt < 4; ++attempt) {
        cb.cand = g->d_cand;
        cb.cand_task = g->d_cand_task;
        cb.cand_cap = (uint32_t)g->cap_cand;
        cb.hits = g->d_hits;
        cb.hit_n = g->d_hit_n;
        CK(cudaMemsetAsync(g->d_ctr, 0, CTR_N * sizeof(unsigned long long), g->stream));
        if (T) cudaEventRecord(g->ev[0], g->stream);
        k_prep<<<(n + 255) / 256, 256, 0, g->stream>>>(cb, g->ix.readlen);
        if (T) cudaEventRecord(g->ev[1], g->stream);
        const uint32_t ntask = n * norient;
        const uint32_t wpb = 4;
        const uint32_t blocks = std::min<uint32_t>((ntask + wpb - 1) / wpb, (uint32_t)g->sm_count * 64);
        if (g->seed_mid_first)
            k_seed_route<<<(ntask + 255) / 256, 256, 0, g->stream>>>(cb, ntask);
        else
            k_seed<<<std::max(1u, blocks), wpb * 32, wpb * LightR::BYTES, g->stream>>>(g->ix, cb, ntask);
        if (T) cudaEventRecord(g->ev[2], g->stream);
        const int tier_launches = seed_tiers(g, cb, g->stream, g->ms, g->hs, T ? g->ev + 7 : nullptr);
        if (T) cudaEventRecord(g->ev[6], g->stream);
        // the automaton widths a read of this index can need (reads shorter than
        // readlen - 20 are invalid, longer than FAME_MAX_READ_LEN refused)
        const uint32_t grid = (uint32_t)g->sm_count * g->sa_blocks_per_sm;
        const uint32_t wlo = std::min(4u, (g->ix.readlen - 20) / 64 + 1);
        if (wlo <= 1) k_shiftand<1><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, FROM_DEVICE);
        if (wlo <= 2) k_shiftand<2><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, FROM_DEVICE);
        if (wlo <= 3) k_shiftand<3><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, FROM_DEVICE);
        k_shiftand<4><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, FROM_DEVICE);
        if (T) cudaEventRecord(g->ev[3], g->stream);
        k_select<<<(n + 255) / 256, 256, 0, g->stream>>>(g->ix, cb);
        if (T) cudaEventRecord(g->ev[4], g->stream);
        k_dp_warp<<<g->dp_blocks, 128, 4 * DPW_BYTES, g->stream>>>(g->ix, cb);
        if (T) cudaEventRecord(g->ev[5], g->stream);
        g->launches += 4 + tier_launches + (int)(5 - wlo);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(g->h_ctr, g->d_ctr, CTR_N * sizeof(unsigned long long), cudaMemcpyDeviceToHost, g->stream));
        CK(cudaStreamSynchronize(g->stream));
        const unsigned long long* h = g->h_ctr;
        if (h[CTR_TOO_LONG]) return set_err(g, FAME_ERR_READ, "read longer than FAME_MAX_READ_LEN");
        if (h[CTR_ERRFLAG]) return set_err(g, FAME_ERR_INDEX, "a device capacity check failed");
        const uint64_t ncand = h[CTR_CAND];
        if (ncand > g->cap_cand) {
            if ((rc = grow_chunk(g, n, 0, ncand + ncand / 4 + 4096))) return rc;
            continue;  // nothing was tallied: redo the chunk with room for all candidates
        }
        if (T) {
            cudaEventElapsedTime(&g->stage_ms[0], g->ev[0], g->ev[1]);
            cudaEventElapsedTime(&g->stage_ms[1], g->ev[1], g->ev[2]);
            cudaEventElapsedTime(&g->stage_ms[5], g->ev[2], g->ev[6]);
            cudaEventElapsedTime(&g->stage_ms[6], g->ev[2], g->ev[7]);
            cudaEventElapsedTime(&g->stage_ms[7], g->ev[7], g->ev[8]);
            cudaEventElapsedTime(&g->stage_ms[8], g->ev[8], g->ev[6]);
            cudaEventElapsedTime(&g->stage_ms[2], g->ev[6], g->ev[3]);
            cudaEventElapsedTime(&g->stage_ms[3], g->ev[3], g->ev[4]);
            cudaEventElapsedTime(&g->stage_ms[4], g->ev[4], g->ev[5]);
        }
        if (cnt) {
            cnt->succ += h[CTR_SUCC];
            cnt->nonunique += h[CTR_NONU];
            cnt->unsucc += h[CTR_UNSUCC];
            cnt->r1_fwd += h[CTR_R1F];
            cnt->r1_rev += h[CTR_R1R];
            cnt->invalid_len += h[CTR_INV_LEN];
            cnt->invalid_n += h[CTR_INV_N];
            cnt->gather_bytes += h[CTR_GATHER_BYTES];
            cnt->windows_scanned += h[CTR_CAND_USED];
            cnt->dp_reads += h[CTR_DP];
            cnt->heavy_tasks += h[CTR_HEAVY];
            cnt->reruns += (uint64_t)attempt;
        }
        {
            // the tasks each tier received: its input list's length
            const unsigned long long* h = g->h_ctr;
            if (g->mid_skip_small) {
                g->tier_tasks[0] = 0;
                g->tier_tasks[1] = h[CTR_HEAVY];
                g->tier_tasks[2] = h[CTR_HEAVY2];
                g->tier_tasks[3] = h[CTR_HEAVY3];
            } else {
                g->tier_tasks[0] = h[CTR_HEAVY];
                g->tier_tasks[1] = h[CTR_HEAVY2];
                g->tier_tasks[2] = h[CTR_HEAVY3];
                g->tier_tasks[3] = h[CTR_HEAVY4];
            }
            g->tier_tasks[4] = h[CTR_REPLAY];
        }
        return FAME_OK;
    }
    return set_err(g, FAME_ERR_NOMEM, "candidate buffer kept overflowing");
}

}  // namespace

extern "C" int fame_gpu_match_reads_dev(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev, uint32_t n,
                                        uint32_t flags, uint64_t* mats_dev, uint8_t* invalid_dev, fame_counters* cnt)
{
    if (!g || (n && (!seqs_dev || !offs_dev || !mats_dev || !invalid_dev))) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    if (n == 0) return FAME_OK;
    return run_chunk(g, seqs_dev, offs_dev, n, flags, mats_dev, invalid_dev, cnt);
}

extern "C" int fame_gpu_match_reads(fame_gpu* g, const char* seqs, const uint64_t* offs, uint32_t n, uint32_t flags,
                                    uint64_t* mats, uint8_t* invalid, fame_counters* cnt)
{
    if (!g || (n && (!seqs || !offs || !mats || !invalid))) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    if (n == 0) return FAME_OK;
    const uint64_t base = offs[0], bytes = offs[n] - offs[0];
    int rc;
    if ((rc = grow_chunk(g, n, bytes, 0))) return rc;
    CK(cudaMemcpyAsync(g->d_seqs, seqs + base, bytes, cudaMemcpyHostToDevice, g->stream));
    if (base == 0) {
        CK(cudaMemcpyAsync(g->d_offs, offs, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, g->stream));
    } else {
        std::vector<uint64_t> o(offs, offs + n + 1);
        for (auto& x : o) x -= base;
        CK(cudaMemcpyAsync(g->d_offs, o.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, g->stream));
        CK(cudaStreamSynchronize(g->stream));
    }
    if ((rc = run_chunk(g, g->d_seqs, g->d_offs, n, flags, g->d_mats, g->d_invalid, cnt))) return rc;
    CK(cudaMemcpyAsync(mats, g->d_mats, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemcpyAsync(invalid, g->d_invalid, n, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    return FAME_OK;
}

namespace {

constexpr uint32_t PE_HEAVY_WARPS = 128;

// Mates of pair r are reads r and n + r of (d_seqs, d_offs); mats and invalid
// hold 2n entries in the same order.
int run_pairs(fame_gpu* g, const char* d_seqs, const uint64_t* d_offs, uint32_t n, uint32_t flags, uint32_t maxpdist,
              uint64_t* d_mats, uint8_t* d_invalid, fame_pair_counters* cnt)
{
    const bool both = flags & FAME_BOTH_STRANDS, stranded = flags & FAME_GET_STRANDED;
    const uint32_t omask = (both || stranded) ? 3u : ((flags & FAME_MATCH_R1_FWD) ? 1u : 2u);
    int rc;
    if ((rc = grow_chunk(g, 2ull * n, 0, 8ull * n + 4096))) return rc;
    if (2ull * n > g->cap_pe_recs) {
        dev_free(g->d_pe_recs);
        const uint64_t c = std::max<uint64_t>(2ull * n, 2048);
        if ((rc = dev_alloc(g, &g->d_pe_recs, c))) return rc;
        g->cap_pe_recs = c;
    }
    if (g->queue) queue_quiesce(g->queue);
    ChunkBufs cb{};
    cb.seqs = d_seqs;
    cb.offs = d_offs;
    cb.n = n;
    cb.orient_mask = omask;
    cb.stranded = stranded ? 1u : 0u;
    cb.rflags = g->d_rflags;
    cb.mats = d_mats;
    cb.invalid = d_invalid;
    cb.dp_list = g->d_dp_list;
    cb.dp_mat = g->d_dp_mat;
    cb.dp_orient = g->d_dp_orient;
    cb.meth = g->d_meth;
    cb.ctr = g->d_ctr;
    cb.heavy = g->d_heavy;
    cb.heavy2 = g->d_heavy2;
    if (!g->d_pe_mid) {
        g->pe_mid_warps = (uint32_t)g->sm_count * 16;   // the register file's limit; 12, 8 and 4 were slower
        g->pe_mid2_warps = (uint32_t)g->sm_count * 4;
        CK(cudaMalloc((void**)&g->d_pe_mid, g->pe_mid_warp_bytes * g->pe_mid_warps));
        CK(cudaMalloc((void**)&g->d_pe_mid2, g->pe_mid2_warp_bytes * g->pe_mid2_warps));
    }
    PeIndex px = g->px;
    px.ctx = (uint32_t)((double)maxpdist / WINLEN) + 1;
    px.maxdist = maxpdist + g->ix.readlen;
    g->launches = 0;
    auto sync_ctr = [&]() -> int {
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(g->h_ctr, g->d_ctr, CTR_N * sizeof(unsigned long long), cudaMemcpyDeviceToHost, g->stream));
        CK(cudaStreamSynchronize(g->stream));
        return FAME_OK;
    };
    for (int attempt = 0; attempt < 4; ++attempt) {
        cb.cand = g->d_cand;
        cb.cand_task = g->d_cand_task;
        cb.cand_flags = g->d_cand_flags;
        cb.cand_cap = (uint32_t)g->cap_cand;
        cb.hits = g->d_hits;
        cb.hit_n = g->d_hit_n;
        cb.cand_first = 0;
        CK(cudaMemsetAsync(g->d_ctr, 0, CTR_N * sizeof(unsigned long long), g->stream));
        const int T = g->timing;
        if (T) cudaEventRecord(g->ev[0], g->stream);
        k_pe_prep<<<(n + 255) / 256, 256, 0, g->stream>>>(cb, g->ix.readlen);
        if (T) cudaEventRecord(g->ev[1], g->stream);
        g->launches++;
        if ((rc = sync_ctr())) return rc;
        if (g->h_ctr[CTR_TOO_LONG]) return set_err(g, FAME_ERR_READ, "mate longer than FAME_MAX_READ_LEN");
        const uint64_t wmask = g->h_ctr[CTR_WMASK];
        // A: maps, walk lists, first-walk candidates; the per-k-mer arrays are
        // sized for the longest valid mate (widths W present: < 64 W bases)
        PeCaps caps = PE_LIGHT;
        {
            uint32_t wmax = 1;
            for (uint32_t w = 1; w <= 4; ++w)
                if ((wmask >> w) & 1u) wmax = w;
            caps.kmax = std::min<uint32_t>(PE_KMAX, 64 * wmax - KMERLEN);
        }
        uint64_t coff[PE_LAYOUT_N];
        const uint64_t wbytes = pe_layout(caps, coff);
        uint32_t grid = g->pe_grid;
        {
            int nb = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pe_seed, 32 * PE_SEED_WARPS,
                                                              PE_SEED_WARPS * wbytes) == cudaSuccess && nb > 0)
                grid = (uint32_t)(g->sm_count * nb);
        }
        k_pe_seed<<<grid, 32 * PE_SEED_WARPS, PE_SEED_WARPS * wbytes, g->stream>>>(g->ix, px, cb, g->d_pe_recs,
                                                                                  (uint32_t)wbytes, caps,
                                                                                  g->seed_mid_first);
        if (T) cudaEventRecord(g->ev[2], g->stream);
        // the paired middle tiers: cb.heavy2 -> (over PE_MID_S) cb.heavy -> (over PE_MID) per-pair path;
        // cb.heavy takes the per-pair path's list only later, in k_pe_finish
        k_pe_seed_mid<<<g->pe_mid_warps / 4, 128, 0, g->stream>>>(g->ix, px, cb, g->d_pe_recs, g->d_pe_mid,
                                                                  g->pe_mid_warp_bytes, PE_MID_S, cb.heavy2,
                                                                  CTR_HEAVY2, CTR_QMID, cb.heavy, CTR_HEAVY3);
        k_pe_seed_mid<<<g->pe_mid2_warps / 4, 128, 0, g->stream>>>(g->ix, px, cb, g->d_pe_recs, g->d_pe_mid2,
                                                                   g->pe_mid2_warp_bytes, PE_MID, cb.heavy,
                                                                   CTR_HEAVY3, CTR_QMID2, nullptr, 0);
        if (T) cudaEventRecord(g->ev[3], g->stream);
        g->launches += 3;
        if ((rc = sync_ctr())) return rc;
        const uint64_t nc1 = g->h_ctr[CTR_CAND];
        if (nc1 > g->cap_cand) {
            if ((rc = grow_chunk(g, 2ull * n, 0, nc1 * 2 + 4096))) return rc;
            continue;
        }
        auto scans = [&](uint64_t first, uint64_t last) {
            if (last <= first) return;
            cb.cand_first = (uint32_t)first;
            const uint32_t grid = (uint32_t)std::min<uint64_t>((last - first + 127) / 128, (uint64_t)g->sm_count * 32);
            if (wmask & 2u) { k_shiftand<1><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, (uint32_t)last); g->launches++; }
            if (wmask & 4u) { k_shiftand<2><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, (uint32_t)last); g->launches++; }
            if (wmask & 8u) { k_shiftand<3><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, (uint32_t)last); g->launches++; }
            if (wmask & 16u) { k_shiftand<4><<<grid, 32 * SA_WARPS, 0, g->stream>>>(g->ix, cb, (uint32_t)last); g->launches++; }
            cb.cand_first = 0;
        };
        // B, C: first-walk scans, first walks, second-walk candidates
        scans(0, nc1);
        if (T) cudaEventRecord(g->ev[4], g->stream);
        k_pe_walk1<<<(2 * n + 127) / 128, 128, 0, g->stream>>>(g->ix, px, cb, g->d_pe_recs);
        if (T) cudaEventRecord(g->ev[5], g->stream);
        g->launches++;
        if ((rc = sync_ctr())) return rc;
        const uint64_t nc2 = g->h_ctr[CTR_CAND];
        if (nc2 > g->cap_cand) {
            if ((rc = grow_chunk(g, 2ull * n, 0, nc2 * 2 + 4096))) return rc;
            continue;
        }
        // D, E: second-walk scans, second walks and the pair choice
        scans(nc1, nc2);
        if (T) cudaEventRecord(g->ev[6], g->stream);
        k_pe_finish<<<(n + 127) / 128, 128, 0, g->stream>>>(g->ix, px, cb, g->d_pe_recs);
        if (T) cudaEventRecord(g->ev[7], g->stream);
        g->launches++;
        if ((rc = sync_ctr())) return rc;
        if (g->h_ctr[CTR_HEAVY]) {
            if (!g->d_pe_heavy) {
                uint64_t off[PE_LAYOUT_N];
                g->pe_heavy_warp_bytes = pe_layout(PE_HEAVY, off);
                g->pe_heavy_warps = PE_HEAVY_WARPS;
                CK(cudaMalloc((void**)&g->d_pe_heavy, g->pe_heavy_warp_bytes * g->pe_heavy_warps));
            }
            k_pe_heavy<<<g->pe_heavy_warps / 4, 128, 0, g->stream>>>(g->ix, px, cb, g->d_pe_heavy,
                                                                      g->pe_heavy_warp_bytes, PE_HEAVY);
            g->launches++;
        }
        k_dp_warp<<<g->dp_grid, 128, 4 * DPW_BYTES, g->stream>>>(g->ix, cb);
        if (T) cudaEventRecord(g->ev[8], g->stream);
        g->launches++;
        if ((rc = sync_ctr())) return rc;
        if (g->h_ctr[CTR_ERRFLAG]) return set_err(g, FAME_ERR_INDEX, "a read pair exceeds the paired path's capacities");
        if (T)
            for (int k = 0; k < FAME_PAIR_STAGES; ++k) cudaEventElapsedTime(&g->pe_stage_ms[k], g->ev[k], g->ev[k + 1]);
        if (cnt) {
            const unsigned long long* h = g->h_ctr;
            cnt->succ += h[CTR_SUCC];
            cnt->nonunique += h[CTR_NONU];
            cnt->unsucc += h[CTR_UNSUCC];
            cnt->paired += h[CTR_PAIRED];
            cnt->too_short += h[CTR_TOOSHORT];
            cnt->r1_fwd += h[CTR_R1F];
            cnt->r1_rev += h[CTR_R1R];
            cnt->dp_reads += h[CTR_DP];
            cnt->heavy_pairs += h[CTR_HEAVY];
        }
        return FAME_OK;
    }
    return set_err(g, FAME_ERR_NOMEM, "candidate buffer kept overflowing");
}

}  // namespace

extern "C" int fame_gpu_match_pairs_dev(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev, uint32_t n,
                                        uint32_t flags, uint32_t maxpdist, uint64_t* mats_dev, uint8_t* invalid_dev,
                                        fame_pair_counters* cnt)
{
    if (!g || (n && (!seqs_dev || !offs_dev || !mats_dev || !invalid_dev))) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    if (n == 0) return FAME_OK;
    return run_pairs(g, seqs_dev, offs_dev, n, flags, maxpdist, mats_dev, invalid_dev, cnt);
}

extern "C" int fame_gpu_match_pairs(fame_gpu* g, const char* seqs1, const uint64_t* offs1, const char* seqs2,
                                    const uint64_t* offs2, uint32_t n, uint32_t flags, uint32_t maxpdist,
                                    uint64_t* mats1, uint64_t* mats2, uint8_t* invalid1, uint8_t* invalid2,
                                    fame_pair_counters* cnt)
{
    if (!g || (n && (!seqs1 || !offs1 || !seqs2 || !offs2 || !mats1 || !mats2 || !invalid1 || !invalid2)))
        return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    if (n == 0) return FAME_OK;
    const uint64_t b1 = offs1[0], n1 = offs1[n] - offs1[0], b2 = offs2[0], n2 = offs2[n] - offs2[0];
    int rc;
    if ((rc = grow_chunk(g, 2ull * n, n1 + n2, 0))) return rc;
    std::vector<uint64_t> o(2ull * n + 1);
    for (uint32_t i = 0; i <= n; ++i) o[i] = offs1[i] - b1;
    for (uint32_t i = 1; i <= n; ++i) o[n + i] = n1 + offs2[i] - b2;
    CK(cudaMemcpyAsync(g->d_seqs, seqs1 + b1, n1, cudaMemcpyHostToDevice, g->stream));
    CK(cudaMemcpyAsync(g->d_seqs + n1, seqs2 + b2, n2, cudaMemcpyHostToDevice, g->stream));
    CK(cudaMemcpyAsync(g->d_offs, o.data(), o.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, g->stream));
    if ((rc = run_pairs(g, g->d_seqs, g->d_offs, n, flags, maxpdist, g->d_mats, g->d_invalid, cnt))) return rc;
    CK(cudaMemcpyAsync(mats1, g->d_mats, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemcpyAsync(mats2, g->d_mats + n, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemcpyAsync(invalid1, g->d_invalid, n, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemcpyAsync(invalid2, g->d_invalid + n, n, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    return FAME_OK;
}

namespace {

// Tallies of a tally array to the host as the reference's uint16 counts
// (packed on the device, one copy), optionally reset; on the context's stream.
int tally_copy_out(fame_gpu* g, uint32_t* meth_dev, uint16_t* meth, int reset)
{
    const uint64_t n4 = 4 * g->n_cpg;
    if (meth && n4) {
        if (!g->d_meth16) {
            int rc;
            if ((rc = dev_alloc(g, &g->d_meth16, n4))) return rc;
        }
        k_pack_tallies<<<g->sm_count * 8, 256, 0, g->stream>>>(meth_dev, n4, g->d_meth16);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(meth, g->d_meth16, n4 * 2, cudaMemcpyDeviceToHost, g->stream));
    }
    if (reset && n4) CK(cudaMemsetAsync(meth_dev, 0, n4 * 4, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    return FAME_OK;
}

}  // namespace

extern "C" int fame_gpu_tallies(fame_gpu* g, uint16_t* meth, int reset)
{
    if (!g) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    return tally_copy_out(g, g->d_meth, meth, reset);
}

extern "C" int fame_gpu_alloc(fame_gpu* g, size_t bytes, void** p)
{
    if (!g || !p) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    CK(cudaMalloc(p, std::max<size_t>(bytes, 16)));
    return FAME_OK;
}

extern "C" int fame_gpu_free(fame_gpu* g, void* p)
{
    if (!g) return FAME_ERR_ARG;
    if (p) CK(cudaFree(p));
    return FAME_OK;
}

extern "C" int fame_gpu_memcpy(fame_gpu* g, void* dst, const void* src, size_t bytes, int kind)
{
    if (!g || (bytes && (!dst || !src))) return FAME_ERR_ARG;
    const cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice : kind == 2 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    CK(cudaMemcpyAsync(dst, src, bytes, k, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    return FAME_OK;
}

extern "C" int fame_gpu_host_alloc(fame_gpu* g, size_t bytes, void** p)
{
    if (!g || !p) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    *p = host_alloc_near(g, bytes);
    if (!*p) return set_err(g, FAME_ERR_NOMEM, "page-locked host allocation");
    return FAME_OK;
}

extern "C" int fame_host_page_node(const void* ptr)
{
    if (!ptr) return -1;
    const uintptr_t pg = (uintptr_t)sysconf(_SC_PAGESIZE);
    void* pages[1] = {(void*)((uintptr_t)ptr & ~(pg - 1))};
    int status[1] = {-1};
    // move_pages without target nodes reports each page's node
    if (syscall(SYS_move_pages, 0, 1ul, pages, nullptr, status, 0) != 0) return -1;
    return status[0] >= 0 ? status[0] : -1;
}

extern "C" int fame_gpu_host_node(fame_gpu* g)
{
    if (!g) return -1;
    int node = -1;
    if (cudaDeviceGetAttribute(&node, cudaDevAttrHostNumaId, g->device) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return node;
}

extern "C" int fame_gpu_host_free(fame_gpu* g, void* p)
{
    if (!g) return FAME_ERR_ARG;
    host_free_near(g, p);
    return FAME_OK;
}

extern "C" int fame_gpu_set_timing(fame_gpu* g, int enable)
{
    if (!g) return FAME_ERR_ARG;
    g->timing = enable;
    return FAME_OK;
}

extern "C" int fame_gpu_stage_times(fame_gpu* g, float* ms, int n)
{
    if (!g || !ms) return FAME_ERR_ARG;
    for (int i = 0; i < n && i < FAME_STAGES; ++i) ms[i] = g->stage_ms[i];
    return FAME_STAGES;
}

extern "C" int fame_gpu_map_order_probe(fame_gpu* g, const uint32_t* keys, uint32_t n, uint32_t bucket_count,
                                        uint32_t* order, uint64_t* final_buckets)
{
    if (!g || (n && (!keys || !order)) || !final_buckets || n > 65536) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    for (uint32_t i = 0; i < n; ++i)
        if (keys[i] >> 31) return set_err(g, FAME_ERR_ARG, "map order probe: keys must leave bit 31 clear");
    const uint32_t cap = 4 * std::max<uint32_t>(n, bucket_count) + 256;
    uint32_t *d_keys = nullptr, *d_scratch = nullptr, *d_order = nullptr, *d_out = nullptr;
    auto done = [&](int rc) {
        dev_free(d_keys); dev_free(d_scratch); dev_free(d_order); dev_free(d_out);
        return rc;
    };
    int rc;
    if ((rc = dev_alloc(g, &d_keys, n)) || (rc = dev_alloc(g, &d_scratch, 3ull * cap)) ||
        (rc = dev_alloc(g, &d_order, n)) || (rc = dev_alloc(g, &d_out, 3)))
        return done(rc);
    uint32_t out[3] = {0, 0, 0};
    if (n && cudaMemcpy(d_keys, keys, 4ull * n, cudaMemcpyHostToDevice) != cudaSuccess)
        return done(set_err(g, FAME_ERR_CUDA, "map order probe: upload"));
    k_map_order_probe<<<1, 32, 0, g->stream>>>(d_keys, n, bucket_count, d_scratch, cap, d_order, d_out);
    if (cudaStreamSynchronize(g->stream) != cudaSuccess ||
        cudaMemcpy(out, d_out, sizeof(out), cudaMemcpyDeviceToHost) != cudaSuccess ||
        (out[0] && cudaMemcpy(order, d_order, 4ull * out[0], cudaMemcpyDeviceToHost) != cudaSuccess))
        return done(set_err(g, FAME_ERR_CUDA, "map order probe failed"));
    if (out[2]) return done(set_err(g, FAME_ERR_INDEX, "map order probe: a capacity was exceeded"));
    *final_buckets = out[1];
    return done((int)out[0]);
}

extern "C" int fame_gpu_pair_stage_times(fame_gpu* g, float* ms, int n)
{
    if (!g || !ms) return FAME_ERR_ARG;
    for (int i = 0; i < n && i < FAME_PAIR_STAGES; ++i) ms[i] = g->pe_stage_ms[i];
    return FAME_PAIR_STAGES;
}

extern "C" int fame_gpu_seed_tier_counts(const fame_gpu* g, uint64_t* out)
{
    if (!g || !out) return FAME_ERR_ARG;
    for (int i = 0; i < 5; ++i) out[i] = g->tier_tasks[i];
    return FAME_OK;
}

extern "C" int fame_gpu_last_launches(const fame_gpu* g) { return g ? g->launches : 0; }

extern "C" uint64_t fame_gpu_index_bytes(const fame_gpu* g) { return g ? g->index_bytes : 0; }

extern "C" int fame_gpu_rec_layout(const fame_gpu* g, uint64_t* slots, uint64_t* nonempty)
{
    if (!g) return FAME_ERR_ARG;
    if (slots) *slots = g->rec_slots;
    if (nonempty) *nonempty = g->nonempty_buckets;
    return g->rec_layout;
}

extern "C" int fame_gpu_set_seed_tier(fame_gpu* g, int mode)
{
    if (!g) return FAME_ERR_ARG;
    if (mode < 0) return g->seed_mid_first + 2 * g->mid_skip_small;
    if (mode > 3) return set_err(g, FAME_ERR_ARG, "seed tier mode must be 0 to 3");
    if (g->queue) queue_drop_graphs(g->queue);
    g->seed_mid_first = mode & 1;
    g->mid_skip_small = (mode >> 1) & 1;
    return FAME_OK;
}

extern "C" int fame_gpu_stream(fame_gpu* g, void** stream)
{
    if (!g || !stream) return FAME_ERR_ARG;
    *stream = (void*)g->stream;
    return FAME_OK;
}

// ---------------------------------------------------------------------------
// CpG calls without any device allocation (fame_gpu_call_cpgs_noalloc).
//
// Some callers of this library cannot allocate device memory while they run:
// a serving loop whose other streams must not be stalled by the device-wide
// synchronisation that cudaFree implies, or code that is only handed buffers
// from an allocator it does not own.  This entry point is a variant of the
// banded-DP CpG kernel (k_dp in kernels.cuh) whose per-read DP matrices live
// in one file-scope static device array instead of context scratch; the
// caller passes its inputs and outputs in device memory it already has.

namespace {

// Layout of the static array: 256 bytes of status counters, then one DP
// matrix (cells) and one alignment trace per slot.  NOALLOC_SLOTS slots serve
// any number of reads (the kernel strides over them); reads up to
// FAME_MAX_READ_LEN bases fit a slot.  Total: about 10.5 MB per GPU.
constexpr uint32_t NOALLOC_SLOTS = 1024;
constexpr uint32_t NOALLOC_CELLS = (FAME_MAX_READ_LEN + 1) * (uint32_t)DPW;
constexpr uint32_t NOALLOC_ALIGN = 2 * FAME_MAX_READ_LEN + 4 * DP_BAND + 8;
constexpr uint64_t NOALLOC_HEADER = 256;
constexpr uint64_t NOALLOC_BYTES =
    NOALLOC_HEADER + (uint64_t)NOALLOC_SLOTS * NOALLOC_CELLS * 2 + (uint64_t)NOALLOC_SLOTS * NOALLOC_ALIGN;
static_assert(CTR_N * sizeof(unsigned long long) <= NOALLOC_HEADER, "status counters exceed the array header");

static __device__ __align__(256) uint8_t g_noalloc_scratch[NOALLOC_BYTES];

__global__ void k_call_cpgs_static(DevIndex ix, ChunkBufs cb, DpScratch ds, const uint64_t* mats, const uint8_t* inval,
                                   uint32_t n, int orient)
{
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= ds.nslots) return;
    for (uint32_t i = slot; i < n; i += ds.nslots) {
        if (inval[i]) continue;
        const uint32_t len = (uint32_t)(cb.offs[i + 1] - cb.offs[i]);
        if (len > FAME_MAX_READ_LEN) { atomicAdd(cb.ctr + CTR_TOO_LONG, 1ull); continue; }
        const uint64_t mat = mats[i];
        const uint32_t meta = (uint32_t)(mat >> 32);
        if (meta >= ix.n_win) { atomicAdd(cb.ctr + CTR_ERRFLAG, 1ull); continue; }
        if (ix.win[meta].z == CPGDUMMY) continue;  // computeMethLvl returns early (ReadQueue.cpp:3287)
        if (((mat >> 16) & 0xff) == 0) meth_exact(ix, cb, i, orient, mat);
        else meth_dp(ix, cb, ds, slot, i, orient, mat);
    }
}

}  // namespace

// The host-side name of the array is only a stand-in: the kernel is given the
// device address, which fame_gpu_open resolves with the device current.
cudaError_t noalloc_scratch_address(void** p) { return cudaGetSymbolAddress(p, g_noalloc_scratch); }

extern "C" int fame_gpu_call_cpgs_noalloc(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev,
                                          const uint64_t* mats_dev, const uint8_t* invalid_dev, uint32_t n,
                                          int orient, uint32_t* meth_dev)
{
    if (!g) return FAME_ERR_ARG;
    if (!meth_dev || (orient != 0 && orient != 1) || (n && (!seqs_dev || !offs_dev || !mats_dev || !invalid_dev)))
        return set_err(g, FAME_ERR_ARG, "fame_gpu_call_cpgs_noalloc: null buffer or orient not 0/1");
    CK(cudaSetDevice(g->device));
    uint8_t* base = g->noalloc_scratch;
    if (!base) return set_err(g, FAME_ERR_CUDA, "no-allocation scratch address unknown");
    cudaStream_t s = g->stream;
    unsigned long long* d_ctr = (unsigned long long*)base;
    CK(cudaMemsetAsync(meth_dev, 0, 16 * g->n_cpg, s));
    CK(cudaMemsetAsync(d_ctr, 0, NOALLOC_HEADER, s));
    if (n) {
        ChunkBufs cb{};
        cb.seqs = seqs_dev;
        cb.offs = offs_dev;
        cb.n = n;
        cb.meth = meth_dev;
        cb.ctr = d_ctr;
        DpScratch ds;
        ds.cells = (uint16_t*)(base + NOALLOC_HEADER);
        ds.align = base + NOALLOC_HEADER + (uint64_t)NOALLOC_SLOTS * NOALLOC_CELLS * 2;
        ds.nslots = NOALLOC_SLOTS;
        ds.cell_cap = NOALLOC_CELLS;
        ds.align_cap = NOALLOC_ALIGN;
        k_call_cpgs_static<<<NOALLOC_SLOTS / 128, 128, 0, s>>>(g->ix, cb, ds, mats_dev, invalid_dev, n,
                                                              orient);
        CK(cudaGetLastError());
    }
    // status counters into this call's own host buffer (pageable, on the
    // stack: no allocation, and nothing shared with the context's other calls)
    unsigned long long h[CTR_N];
    CK(cudaMemcpyAsync(h, d_ctr, CTR_N * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h[CTR_TOO_LONG]) return set_err(g, FAME_ERR_READ, "a read is longer than FAME_MAX_READ_LEN");
    if (h[CTR_ERRFLAG]) return set_err(g, FAME_ERR_ARG, "a match names no window of the index");
    return FAME_OK;
}

#include "queue.cuh"
#include "tune.cuh"

void queue_quiesce(fame_queue* q)
{
    for (auto& s : q->slots)
        if (s.stream) cudaStreamSynchronize(s.stream);
}

void queue_drop_graphs(fame_queue* q)
{
    queue_quiesce(q);
    for (auto& s : q->slots) {
        for (auto& gr : s.graphs) cudaGraphExecDestroy(gr.exec);
        s.graphs.clear();
    }
}
