// Autotuner of the chunk pipeline's launch shapes (no counterpart in the
// reference).  It times the stages on a sample chunk the caller provides and
// keeps, stage by stage, the fastest of a few shapes:
//
//   seed_mode         where seeding starts, and whether the shared-memory
//                     middle tiers start at the smaller or the larger one
//                     (fame_gpu_set_seed_tier: 0..3)
//   sa_blocks_per_sm  k_shiftand blocks per SM (its warps loop over the
//                     candidates, 32 at a time)
//   dp_blocks_per_sm  k_dp_warp blocks per SM (up to its occupancy; three
//                     reads per warp, the warps loop over the DP list)
//
// A shape changes how work is spread over the GPU, never what is computed:
// every trial's per-read results are compared with the first trial's and a
// difference is an error.  The choice is written as a small JSON file and
// can be loaded again with fame_gpu_load_tuning.
//
// Included into fame_gpu.cu (it drives run_chunk).

#include <cstdlib>
#include <fstream>
#include <sstream>

namespace {

struct TuneShape {
    int seed_mode;
    uint32_t sa_blocks_per_sm;
    uint32_t dp_blocks_per_sm;
};

void tune_apply(fame_gpu* g, const TuneShape& t)
{
    if (g->queue) queue_drop_graphs(g->queue);   // graphs captured with the old shapes
    g->seed_mid_first = t.seed_mode & 1;
    g->mid_skip_small = (t.seed_mode >> 1) & 1;
    g->sa_blocks_per_sm = t.sa_blocks_per_sm;
    g->dp_blocks = std::max<uint32_t>(1, std::min<uint32_t>(g->dp_grid, t.dp_blocks_per_sm * (uint32_t)g->sm_count));
}

TuneShape tune_current(const fame_gpu* g)
{
    return TuneShape{g->seed_mid_first + 2 * g->mid_skip_small, g->sa_blocks_per_sm,
                     std::max<uint32_t>(1, g->dp_blocks / (uint32_t)g->sm_count)};
}

}  // namespace

extern "C" int fame_gpu_autotune(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev, uint32_t n,
                                 uint32_t flags, const char* json_path)
{
    if (!g || !seqs_dev || !offs_dev || n == 0) return FAME_ERR_ARG;
    CK(cudaSetDevice(g->device));
    const TuneShape start = tune_current(g);
    uint64_t* d_mats = nullptr;
    uint8_t* d_inv = nullptr;
    uint32_t* d_meth = nullptr;
    std::vector<uint64_t> ref_mats(n), mats(n);
    std::vector<uint8_t> ref_inv(n), inv(n);
    bool have_ref = false;
    const int saved_timing = g->timing;
    std::ostringstream trials;
    auto cleanup = [&]() {
        if (d_mats) cudaFree(d_mats);
        if (d_inv) cudaFree(d_inv);
        if (d_meth) cudaFree(d_meth);
        g->timing = saved_timing;
    };
    // the trials tally into their own array, so the context's tallies stay as they were
    if (cudaMalloc((void**)&d_mats, 8ull * n) != cudaSuccess || cudaMalloc((void**)&d_inv, n) != cudaSuccess ||
        cudaMalloc((void**)&d_meth, 16 * std::max<uint64_t>(1, g->n_cpg)) != cudaSuccess) {
        cleanup();
        return set_err(g, FAME_ERR_NOMEM, "autotune scratch allocation failed");
    }
    g->timing = 1;
    // one trial: the chunk twice (the first warms caches and grows buffers),
    // the stage times of the second, results checked against the first trial
    auto trial = [&](const TuneShape& t, float* ms) -> int {
        tune_apply(g, t);
        for (int rep = 0; rep < 2; ++rep) {
            fame_counters c{};
            const int r = run_chunk(g, seqs_dev, offs_dev, n, flags, d_mats, d_inv, &c, d_meth);
            if (r) return r;
        }
        for (int k = 0; k < FAME_STAGES; ++k) ms[k] = g->stage_ms[k];
        CK(cudaMemcpy(mats.data(), d_mats, 8ull * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(inv.data(), d_inv, n, cudaMemcpyDeviceToHost));
        if (!have_ref) {
            ref_mats = mats;
            ref_inv = inv;
            have_ref = true;
        } else if (mats != ref_mats || inv != ref_inv) {
            return set_err(g, FAME_ERR_INDEX, "autotune: results differ between launch shapes");
        }
        trials << (trials.tellp() > 0 ? ",\n    " : "") << "{\"seed_mode\": " << t.seed_mode
               << ", \"sa_blocks_per_sm\": " << t.sa_blocks_per_sm << ", \"dp_blocks_per_sm\": " << t.dp_blocks_per_sm
               << ", \"stage_ms\": [";
        for (int k = 0; k < FAME_STAGES; ++k) trials << (k ? ", " : "") << ms[k];
        trials << "]}";
        return FAME_OK;
    };
    int rc = FAME_OK;
    TuneShape best = start;
    float ms[FAME_STAGES];
    // seeding: stages 1 (light tier or routing) and 5 (the other tiers)
    {
        float best_t = 1e30f;
        for (int mode = 0; mode < 4 && !rc; ++mode) {
            TuneShape t = best;
            t.seed_mode = mode;
            if ((rc = trial(t, ms))) break;
            if (ms[1] + ms[5] < best_t) { best_t = ms[1] + ms[5]; best.seed_mode = mode; }
        }
    }
    // window scans: stage 2
    if (!rc) {
        float best_t = 1e30f;
        for (uint32_t b : {8u, 16u, 32u}) {
            TuneShape t = best;
            t.sa_blocks_per_sm = b;
            if ((rc = trial(t, ms))) break;
            if (ms[2] < best_t) { best_t = ms[2]; best.sa_blocks_per_sm = b; }
        }
    }
    // banded DP: stage 4
    if (!rc) {
        float best_t = 1e30f;
        const uint32_t occ = std::max<uint32_t>(1, g->dp_grid / (uint32_t)g->sm_count);
        for (uint32_t b : {std::max(1u, occ / 2), occ}) {
            TuneShape t = best;
            t.dp_blocks_per_sm = b;
            if ((rc = trial(t, ms))) break;
            if (ms[4] < best_t) { best_t = ms[4]; best.dp_blocks_per_sm = b; }
        }
    }
    cleanup();
    if (rc) {
        tune_apply(g, start);
        return rc;
    }
    tune_apply(g, best);
    if (json_path && *json_path) {
        std::ofstream f(json_path, std::ios::trunc);
        f << "{\n  \"seed_mode\": " << best.seed_mode << ",\n  \"sa_blocks_per_sm\": " << best.sa_blocks_per_sm
          << ",\n  \"dp_blocks_per_sm\": " << best.dp_blocks_per_sm << ",\n  \"sample_reads\": " << n
          << ",\n  \"flags\": " << flags << ",\n  \"sm_count\": " << g->sm_count
          << ",\n  \"stages\": [\"read_prep\", \"seed\", \"shift_and\", \"select\", \"banded_dp\", \"seed_tiers\", "
             "\"seed_mid_small\", \"seed_mid_large\", \"seed_global\"],"
          << "\n  \"trials\": [\n    " << trials.str() << "\n  ]\n}\n";
        if (!f) return set_err(g, FAME_ERR_IO, std::string("autotune: cannot write ") + json_path);
    }
    return FAME_OK;
}

extern "C" int fame_gpu_load_tuning(fame_gpu* g, const char* json_path)
{
    if (!g || !json_path) return FAME_ERR_ARG;
    std::ifstream f(json_path);
    if (!f) return set_err(g, FAME_ERR_IO, std::string("cannot read ") + json_path);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    // the three top-level keys, written first by fame_gpu_autotune
    auto get = [&](const char* key, long* out) -> bool {
        const std::string k = std::string("\"") + key + "\"";
        const size_t p = t.find(k);
        if (p == std::string::npos) return false;
        const size_t c = t.find(':', p + k.size());
        if (c == std::string::npos) return false;
        char* end = nullptr;
        *out = std::strtol(t.c_str() + c + 1, &end, 10);
        return end != t.c_str() + c + 1;
    };
    long mode = 0, sa = 0, dp = 0;
    if (!get("seed_mode", &mode) || !get("sa_blocks_per_sm", &sa) || !get("dp_blocks_per_sm", &dp) || mode < 0 ||
        mode > 3 || sa < 1 || sa > 64 || dp < 1 || dp > 64)
        return set_err(g, FAME_ERR_IO, std::string("not a tuning file: ") + json_path);
    tune_apply(g, TuneShape{(int)mode, (uint32_t)sa, (uint32_t)dp});
    return FAME_OK;
}
