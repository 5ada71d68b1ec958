// Batched / serving form: a queue of chunk slots on one context.
//
// Each slot owns the device buffers of one chunk, page-locked staging for its
// inputs and outputs, a CUDA stream and a cache of CUDA graphs.  A submitted
// chunk is copied into the slot (host memcpy into the staging buffers, then
// asynchronous copies to the device) and the chunk pipeline runs as one
// captured graph with no host round trip inside: the kernels read the
// candidate, heavy-task and automaton-width counts from the chunk's device
// counters (FROM_DEVICE), launch every automaton width (a width without reads
// returns at once) and stop after seeding when the candidate buffer
// overflowed.  Chunks in different slots overlap on the GPU.  Collecting a
// chunk waits for its event; an overflowed chunk is rerun through the plain
// path, after the other slots are idle (that path uses the context's shared
// scratch), with the same tally array.
//
// The graph of a slot depends on the chunk's read count, flags and tally
// array; graphs are cached per slot (up to 8 shapes).
//
// Included into fame_gpu.cu (one translation unit for all kernels).

#include <chrono>
#include <thread>

namespace {

constexpr uint32_t QUEUE_GRAPHS = 8;

struct QSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    // device
    char* d_seqs = nullptr;
    uint64_t* d_offs = nullptr;
    uint8_t* d_rflags = nullptr;
    uint4* d_task_cand = nullptr;
    uint32_t *d_cand = nullptr, *d_cand_task = nullptr, *d_hits = nullptr, *d_hit_n = nullptr;
    uint64_t* d_mats = nullptr;
    uint8_t* d_invalid = nullptr;
    uint32_t* d_dp_list = nullptr;
    uint64_t* d_dp_mat = nullptr;
    uint8_t* d_dp_orient = nullptr;
    uint32_t* d_heavy = nullptr;
    uint32_t* d_heavy2 = nullptr;
    unsigned long long* d_ctr = nullptr;
    // page-locked staging
    char* h_seqs = nullptr;
    uint64_t* h_offs = nullptr;
    uint64_t* h_mats = nullptr;
    uint8_t* h_invalid = nullptr;
    unsigned long long* h_ctr = nullptr;
    HeavyScratch hs{};      // this slot's part of the context's large-capacity tier
    HeavyScratch ms{};      // and of its middle tier
    uint64_t cap_cand = 0;
    // the chunk in flight
    bool busy = false;
    uint32_t n = 0;
    uint32_t flags = 0;
    uint32_t* meth = nullptr;
    bool staged = false;       // handed to the caller by fame_queue_stage, not yet submitted
    // graph cache
    struct Graph {
        uint32_t n, flags;
        uint32_t* meth;
        cudaGraphExec_t exec;
        uint64_t used;
    };
    std::vector<Graph> graphs;
};

}  // namespace

struct fame_queue {
    fame_gpu* g = nullptr;
    std::vector<QSlot> slots;
    uint32_t max_reads = 0;
    uint64_t max_bytes = 0;
    uint64_t tick = 0;
    uint64_t launches = 0;
};

namespace {

void qslot_free(fame_gpu* g, QSlot& s)
{
    for (auto& gr : s.graphs) cudaGraphExecDestroy(gr.exec);
    s.graphs.clear();
    dev_free(s.d_seqs); dev_free(s.d_offs); dev_free(s.d_rflags); dev_free(s.d_task_cand); dev_free(s.d_cand);
    dev_free(s.d_cand_task); dev_free(s.d_hits); dev_free(s.d_hit_n); dev_free(s.d_mats); dev_free(s.d_invalid);
    dev_free(s.d_dp_list); dev_free(s.d_dp_mat); dev_free(s.d_dp_orient); dev_free(s.d_heavy); dev_free(s.d_heavy2); dev_free(s.d_ctr);
    host_free_near(g, s.h_seqs);
    host_free_near(g, s.h_offs);
    host_free_near(g, s.h_mats);
    host_free_near(g, s.h_invalid);
    if (s.h_ctr) cudaFreeHost(s.h_ctr);
    s.h_seqs = nullptr; s.h_offs = nullptr; s.h_mats = nullptr; s.h_invalid = nullptr; s.h_ctr = nullptr;
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
    s.done = nullptr;
    s.stream = nullptr;
}

ChunkBufs qslot_bufs(fame_gpu* g, QSlot& s, uint32_t n, uint32_t flags, uint32_t* meth)
{
    const bool both = flags & FAME_BOTH_STRANDS, stranded = flags & FAME_GET_STRANDED;
    ChunkBufs cb{};
    cb.seqs = s.d_seqs;
    cb.offs = s.d_offs;
    cb.n = n;
    cb.orient_mask = (both || stranded) ? 3u : ((flags & FAME_MATCH_R1_FWD) ? 1u : 2u);
    cb.stranded = stranded ? 1u : 0u;
    cb.rflags = s.d_rflags;
    cb.task_cand = s.d_task_cand;
    cb.cand = s.d_cand;
    cb.cand_task = s.d_cand_task;
    cb.cand_cap = (uint32_t)s.cap_cand;
    cb.hits = s.d_hits;
    cb.hit_n = s.d_hit_n;
    cb.mats = s.d_mats;
    cb.invalid = s.d_invalid;
    cb.dp_list = s.d_dp_list;
    cb.dp_mat = s.d_dp_mat;
    cb.dp_orient = s.d_dp_orient;
    cb.meth = meth ? meth : g->d_meth;
    cb.ctr = s.d_ctr;
    cb.heavy = s.d_heavy;
    cb.heavy2 = s.d_heavy2;
    return cb;
}

// The kernels of one chunk, with every count read on the device.
void qslot_enqueue(fame_gpu* g, QSlot& s, uint32_t n, uint32_t flags, uint32_t* meth)
{
    const ChunkBufs cb = qslot_bufs(g, s, n, flags, meth);
    const uint32_t norient = cb.orient_mask == 3u ? 2u : 1u;
    cudaMemsetAsync(s.d_ctr, 0, CTR_N * sizeof(unsigned long long), s.stream);
    k_prep<<<(n + 255) / 256, 256, 0, s.stream>>>(cb, g->ix.readlen);
    const uint32_t ntask = n * norient;
    const uint32_t blocks = std::min<uint32_t>((ntask + 3) / 4, (uint32_t)g->sm_count * 64);
    if (g->seed_mid_first)
        k_seed_route<<<(ntask + 255) / 256, 256, 0, s.stream>>>(cb, ntask);
    else
        k_seed<<<std::max(1u, blocks), 128, 4 * LightR::BYTES, s.stream>>>(g->ix, cb, ntask);
    seed_tiers(g, cb, s.stream, s.ms, s.hs);
    const uint32_t grid = (uint32_t)g->sm_count * g->sa_blocks_per_sm;
    k_shiftand<1><<<grid, 32 * SA_WARPS, 0, s.stream>>>(g->ix, cb, FROM_DEVICE);
    k_shiftand<2><<<grid, 32 * SA_WARPS, 0, s.stream>>>(g->ix, cb, FROM_DEVICE);
    k_shiftand<3><<<grid, 32 * SA_WARPS, 0, s.stream>>>(g->ix, cb, FROM_DEVICE);
    k_shiftand<4><<<grid, 32 * SA_WARPS, 0, s.stream>>>(g->ix, cb, FROM_DEVICE);
    k_select<<<(n + 255) / 256, 256, 0, s.stream>>>(g->ix, cb);
    k_dp_warp<<<g->dp_blocks, 128, 4 * DPW_BYTES, s.stream>>>(g->ix, cb);
    cudaMemcpyAsync(s.h_mats, s.d_mats, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, s.stream);
    cudaMemcpyAsync(s.h_invalid, s.d_invalid, n, cudaMemcpyDeviceToHost, s.stream);
    cudaMemcpyAsync(s.h_ctr, s.d_ctr, CTR_N * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s.stream);
}

constexpr uint64_t QUEUE_KERNELS_PER_CHUNK = 13;

int qslot_graph(fame_gpu* g, fame_queue* q, QSlot& s, uint32_t n, uint32_t flags, uint32_t* meth, cudaGraphExec_t* out)
{
    for (auto& gr : s.graphs)
        if (gr.n == n && gr.flags == flags && gr.meth == meth) {
            gr.used = ++q->tick;
            *out = gr.exec;
            return FAME_OK;
        }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
    qslot_enqueue(g, s, n, flags, meth);
    const cudaError_t e1 = cudaGetLastError();
    const cudaError_t e2 = cudaStreamEndCapture(s.stream, &graph);
    if (e1 != cudaSuccess || e2 != cudaSuccess)
        return set_err(g, FAME_ERR_CUDA, std::string("chunk graph capture: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    cudaGraphExec_t exec;
    const cudaError_t e3 = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) return set_err(g, FAME_ERR_CUDA, std::string("chunk graph instantiate: ") + cudaGetErrorString(e3));
    if (s.graphs.size() >= QUEUE_GRAPHS) {
        auto old = std::min_element(s.graphs.begin(), s.graphs.end(),
                                    [](const QSlot::Graph& a, const QSlot::Graph& b) { return a.used < b.used; });
        cudaGraphExecDestroy(old->exec);
        s.graphs.erase(old);
    }
    s.graphs.push_back({n, flags, meth, exec, ++q->tick});
    *out = exec;
    return FAME_OK;
}

}  // namespace

extern "C" int fame_queue_open(fame_gpu* g, uint32_t nslots, uint32_t max_reads, uint64_t max_bytes, fame_queue** out)
{
    if (!g || !out || nslots == 0 || nslots > 8 || max_reads == 0 || max_bytes == 0) return FAME_ERR_ARG;
    if (g->queue) return set_err(g, FAME_ERR_BUSY, "the context already has a queue");
    *out = nullptr;
    CK(cudaSetDevice(g->device));
    fame_queue* q = new (std::nothrow) fame_queue();
    if (!q) return FAME_ERR_NOMEM;
    q->g = g;
    q->max_reads = max_reads;
    q->max_bytes = max_bytes;
    q->slots.resize(nslots);
    const uint64_t cand = 2ull * max_reads * 4 + 4096;
    const uint32_t hw = std::max(1u, g->hs.nwarps / nslots);
    auto fail = [&](int rc) {
        for (auto& s : q->slots) qslot_free(g, s);
        delete q;
        return rc;
    };
    for (uint32_t i = 0; i < nslots; ++i) {
        QSlot& s = q->slots[i];
        int rc;
        if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_CUDA, "queue stream"));
        if ((rc = dev_alloc(g, &s.d_seqs, max_bytes)) || (rc = dev_alloc(g, &s.d_offs, max_reads + 1ull)) ||
            (rc = dev_alloc(g, &s.d_rflags, max_reads)) || (rc = dev_alloc(g, &s.d_task_cand, 2ull * max_reads)) ||
            (rc = dev_alloc(g, &s.d_cand, cand)) || (rc = dev_alloc(g, &s.d_cand_task, cand)) ||
            (rc = dev_alloc(g, &s.d_hits, cand * HIT_CAP)) || (rc = dev_alloc(g, &s.d_hit_n, cand)) ||
            (rc = dev_alloc(g, &s.d_mats, max_reads)) || (rc = dev_alloc(g, &s.d_invalid, max_reads)) ||
            (rc = dev_alloc(g, &s.d_dp_list, max_reads)) || (rc = dev_alloc(g, &s.d_dp_mat, max_reads)) ||
            (rc = dev_alloc(g, &s.d_dp_orient, max_reads)) || (rc = dev_alloc(g, &s.d_heavy, 2ull * max_reads)) ||
            (rc = dev_alloc(g, &s.d_heavy2, 2ull * max_reads)) ||
            (rc = dev_alloc(g, &s.d_ctr, CTR_N)))
            return fail(rc);
        s.h_seqs = (char*)host_alloc_near(g, max_bytes);
        s.h_offs = (uint64_t*)host_alloc_near(g, (max_reads + 1ull) * 8);
        s.h_mats = (uint64_t*)host_alloc_near(g, max_reads * 8ull);
        s.h_invalid = (uint8_t*)host_alloc_near(g, max_reads);
        if (!s.h_seqs || !s.h_offs || !s.h_mats || !s.h_invalid ||
            cudaMallocHost((void**)&s.h_ctr, CTR_N * sizeof(unsigned long long)) != cudaSuccess)
            return fail(set_err(g, FAME_ERR_NOMEM, "queue page-locked staging"));
        s.cap_cand = cand;
        // each slot takes its own share of the heavy-path scratch
        s.hs = g->hs;
        s.hs.nwarps = hw;
        s.hs.base = g->hs.base + (uint64_t)i * hw * g->hs.bytes_per_warp;   // nslots <= 8 <= hs.nwarps
        s.ms = g->ms;
        s.ms.nwarps = std::max(1u, g->ms.nwarps / nslots);
        s.ms.base = g->ms.base + (uint64_t)i * s.ms.nwarps * g->ms.bytes_per_warp;
    }
    g->queue = q;
    *out = q;
    return FAME_OK;
}

namespace {

int qslot_free_index(fame_queue* q)
{
    for (size_t i = 0; i < q->slots.size(); ++i)
        if (!q->slots[i].busy && !q->slots[i].staged) return (int)i;
    return -1;
}

// The chunk in slot pick's staging (s.h_seqs / s.h_offs, offsets from 0):
// copies, the cached graph, the completion event.
int qslot_launch(fame_queue* q, int pick, uint32_t n, uint32_t flags, uint32_t* meth_dev, int* slot)
{
    fame_gpu* g = q->g;
    QSlot& s = q->slots[pick];
    const uint64_t bytes = n ? s.h_offs[n] : 0;
    s.n = n;
    s.flags = flags;
    s.meth = meth_dev;
    s.busy = true;
    if (n == 0) {
        std::memset(s.h_ctr, 0, CTR_N * sizeof(unsigned long long));
        CK(cudaEventRecord(s.done, s.stream));
        *slot = pick;
        return FAME_OK;
    }
    CK(cudaMemcpyAsync(s.d_seqs, s.h_seqs, std::max<uint64_t>(bytes, 1), cudaMemcpyHostToDevice, s.stream));
    CK(cudaMemcpyAsync(s.d_offs, s.h_offs, (n + 1ull) * 8, cudaMemcpyHostToDevice, s.stream));
    cudaGraphExec_t exec;
    int rc;
    if ((rc = qslot_graph(g, q, s, n, flags, meth_dev, &exec))) { s.busy = false; return rc; }
    CK(cudaGraphLaunch(exec, s.stream));
    CK(cudaEventRecord(s.done, s.stream));
    q->launches += QUEUE_KERNELS_PER_CHUNK;
    *slot = pick;
    return FAME_OK;
}

}  // namespace

extern "C" int fame_queue_submit(fame_queue* q, const char* seqs, const uint64_t* offs, uint32_t n, uint32_t flags,
                                 uint32_t* meth_dev, int* slot)
{
    if (!q || !slot || (n && (!seqs || !offs))) return FAME_ERR_ARG;
    fame_gpu* g = q->g;
    if (n > q->max_reads || (n && offs[n] - offs[0] > q->max_bytes))
        return set_err(g, FAME_ERR_ARG, "chunk exceeds the queue's slot size");
    CK(cudaSetDevice(g->device));
    const int pick = qslot_free_index(q);
    if (pick < 0) return set_err(g, FAME_ERR_BUSY, "every queue slot holds an uncollected chunk");
    QSlot& s = q->slots[pick];
    const uint64_t base = n ? offs[0] : 0, bytes = n ? offs[n] - offs[0] : 0;
    std::memcpy(s.h_seqs, seqs + base, bytes);
    for (uint32_t i = 0; i <= n; ++i) s.h_offs[i] = n ? offs[i] - base : 0;
    return qslot_launch(q, pick, n, flags, meth_dev, slot);
}

extern "C" int fame_queue_stage(fame_queue* q, int* slot, char** seqs, uint64_t** offs, uint32_t* max_reads,
                                uint64_t* max_bytes)
{
    if (!q || !slot || !seqs || !offs) return FAME_ERR_ARG;
    const int pick = qslot_free_index(q);
    if (pick < 0) return set_err(q->g, FAME_ERR_BUSY, "every queue slot holds an uncollected chunk");
    QSlot& s = q->slots[pick];
    s.staged = true;
    *slot = pick;
    *seqs = s.h_seqs;
    *offs = s.h_offs;
    if (max_reads) *max_reads = q->max_reads;
    if (max_bytes) *max_bytes = q->max_bytes;
    return FAME_OK;
}

extern "C" int fame_queue_submit_staged(fame_queue* q, int slot, uint32_t n, uint32_t flags, uint32_t* meth_dev)
{
    if (!q || slot < 0 || slot >= (int)q->slots.size()) return FAME_ERR_ARG;
    fame_gpu* g = q->g;
    QSlot& s = q->slots[slot];
    if (!s.staged) return set_err(g, FAME_ERR_ARG, "queue slot was not staged");
    s.staged = false;
    if (n > q->max_reads || (n && (s.h_offs[0] != 0 || s.h_offs[n] > q->max_bytes)))
        return set_err(g, FAME_ERR_ARG, "staged chunk exceeds the queue's slot size");
    CK(cudaSetDevice(g->device));
    int out = 0;
    return qslot_launch(q, slot, n, flags, meth_dev, &out);
}

extern "C" int fame_queue_ready(fame_queue* q, int slot)
{
    if (!q || slot < 0 || slot >= (int)q->slots.size()) return FAME_ERR_ARG;
    const QSlot& s = q->slots[slot];
    if (!s.busy) return 0;
    return cudaEventQuery(s.done) == cudaSuccess ? 1 : 0;
}

extern "C" int fame_queue_wait(fame_queue* q, int slot, uint32_t timeout_ms)
{
    if (!q || slot < 0 || slot >= (int)q->slots.size()) return FAME_ERR_ARG;
    const QSlot& s = q->slots[slot];
    if (!s.busy) return FAME_OK;
    // poll with a deadline instead of blocking in cudaEventSynchronize
    const auto t0 = std::chrono::steady_clock::now();
    while (true) {
        const cudaError_t e = cudaEventQuery(s.done);
        if (e == cudaSuccess) return FAME_OK;
        if (e != cudaErrorNotReady)
            return set_err(q->g, FAME_ERR_CUDA, std::string("queue slot wait: ") + cudaGetErrorString(e));
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (ms >= (double)timeout_ms) return FAME_ERR_TIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

extern "C" int fame_queue_collect(fame_queue* q, int slot, uint64_t* mats, uint8_t* invalid, fame_counters* cnt)
{
    if (!q || slot < 0 || slot >= (int)q->slots.size()) return FAME_ERR_ARG;
    QSlot& s = q->slots[slot];
    fame_gpu* g = q->g;
    if (!s.busy) return set_err(g, FAME_ERR_ARG, "queue slot holds no chunk");
    CK(cudaSetDevice(g->device));
    CK(cudaEventSynchronize(s.done));
    s.busy = false;
    const unsigned long long* h = s.h_ctr;
    if (h[CTR_TOO_LONG]) return set_err(g, FAME_ERR_READ, "read longer than FAME_MAX_READ_LEN");
    if (h[CTR_ERRFLAG]) return set_err(g, FAME_ERR_INDEX, "a device capacity check failed");
    if (h[CTR_CAND] > s.cap_cand) {
        // rerun through the plain path (its buffers grow to fit); nothing was tallied
        int rc = run_chunk(g, s.d_seqs, s.d_offs, s.n, s.flags, s.d_mats, s.d_invalid, cnt, s.meth);
        if (rc) return rc;
        if (cnt) cnt->reruns += 1;
        if (mats) CK(cudaMemcpy(mats, s.d_mats, s.n * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        if (invalid) CK(cudaMemcpy(invalid, s.d_invalid, s.n, cudaMemcpyDeviceToHost));
        return FAME_OK;
    }
    if (mats) std::memcpy(mats, s.h_mats, s.n * sizeof(uint64_t));
    if (invalid) std::memcpy(invalid, s.h_invalid, s.n);
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
    }
    return FAME_OK;
}

extern "C" uint64_t fame_queue_launches(const fame_queue* q) { return q ? q->launches : 0; }

extern "C" int fame_queue_close(fame_queue* q)
{
    if (!q) return FAME_ERR_ARG;
    cudaSetDevice(q->g->device);
    for (auto& s : q->slots) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        qslot_free(q->g, s);
    }
    q->g->queue = nullptr;
    delete q;
    return FAME_OK;
}

extern "C" int fame_gpu_tally_alloc(fame_gpu* g, uint32_t** meth_dev)
{
    if (!g || !meth_dev) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    const uint64_t bytes = 16 * std::max<uint64_t>(1, g->n_cpg);
    CK(cudaMalloc((void**)meth_dev, bytes));
    CK(cudaMemset(*meth_dev, 0, bytes));
    return FAME_OK;
}

extern "C" int fame_gpu_tally_read(fame_gpu* g, const uint32_t* meth_dev, uint16_t* meth, int reset)
{
    if (!g || !meth_dev) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    return tally_copy_out(g, (uint32_t*)meth_dev, meth, reset);
}

extern "C" int fame_gpu_tally_free(fame_gpu* g, uint32_t* meth_dev)
{
    if (!g) return FAME_ERR_ARG;
    if (meth_dev) CK(cudaFree(meth_dev));
    return FAME_OK;
}

extern "C" int fame_gpu_mem_info(fame_gpu* g, uint64_t* free_bytes, uint64_t* total_bytes)
{
    if (!g || !free_bytes || !total_bytes) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    size_t f = 0, t = 0;
    CK(cudaMemGetInfo(&f, &t));
    *free_bytes = f;
    *total_bytes = t;
    return FAME_OK;
}
