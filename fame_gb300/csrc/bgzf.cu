// BGZF input inflated on the GPU: one warp per gzip member (at most 64 KiB
// of output each), the DEFLATE decoder and CRC-32 of inflate.h.  The FASTQ
// reader finds the members on the host (their compressed and uncompressed
// sizes are in each member's header and trailer), so the outputs are laid out
// before the launch and the threads need no coordination.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <vector>

#include "../../include/fame_gpu.h"
#include "bgzf.h"
#include "inflate.h"

namespace fame {

namespace {

constexpr uint32_t BGZF_WARPS = 4;   // warps per block, one member each

// One warp per member: every lane runs the decoder on the same member in
// step (the same loads, branches and stores: no divergence, one transaction
// per store), the warp's code tables in shared memory.  One thread per
// member would put 32 unrelated bit streams in a warp and serialise them.
__global__ void __launch_bounds__(32 * BGZF_WARPS) k_bgzf_inflate(const uint8_t* comp, const BgzfMember* m, uint32_t n,
                                                                  uint8_t* out, uint32_t* status)
{
    __shared__ uint32_t crc_t[256];
    __shared__ InflScratch sc[BGZF_WARPS];
    for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) {
        uint32_t c = i;
        for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        crc_t[i] = c;
    }
    __syncthreads();
    const uint32_t wib = threadIdx.x >> 5;
    const uint32_t i = blockIdx.x * BGZF_WARPS + wib;
    if (i >= n) return;
    const BgzfMember mm = m[i];
    uint32_t got = 0;
    int r = infl_raw(comp + mm.coff, mm.clen, out + mm.ooff, mm.isize, &got, sc[wib]);
    if (r == INFL_OK && got != mm.isize) r = INFL_ERR_SIZE;
    if (r == INFL_OK && crc32_of(crc_t, out + mm.ooff, got) != mm.crc) r = INFL_ERR_CRC;
    if ((threadIdx.x & 31) == 0) status[i] = (uint32_t)r;
}

}  // namespace

struct BgzfGpu {
    int dev = 0;
    cudaStream_t st = nullptr;
    uint8_t* d_comp = nullptr;
    uint64_t comp_cap = 0;
    uint8_t* d_out = nullptr;
    uint64_t out_cap = 0;
    BgzfMember* d_m = nullptr;
    uint64_t m_cap = 0;
    uint32_t* d_status = nullptr;
    uint64_t status_cap = 0;
    std::vector<uint32_t> status;
};

BgzfGpu* bgzf_gpu_open(int device)
{
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess) return nullptr;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    BgzfGpu* b = new (std::nothrow) BgzfGpu();
    if (b) {
        b->dev = device;
        if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            delete b;
            b = nullptr;
        }
    }
    cudaSetDevice(prev);
    return b;
}

void bgzf_gpu_close(BgzfGpu* b)
{
    if (!b) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->dev);
    if (b->st) cudaStreamSynchronize(b->st);
    cudaFree(b->d_comp);
    cudaFree(b->d_out);
    cudaFree(b->d_m);
    cudaFree(b->d_status);
    if (b->st) cudaStreamDestroy(b->st);
    cudaSetDevice(prev);
    delete b;
}

int bgzf_gpu_inflate(BgzfGpu* b, const uint8_t* comp, uint64_t comp_len, const BgzfMember* m, uint32_t n,
                     uint8_t* out, uint64_t out_len)
{
    if (!b) return FAME_ERR_ARG;
    if (n == 0) return FAME_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(b->dev) != cudaSuccess) return FAME_ERR_CUDA;
    int rc = FAME_OK;
    auto grow = [&](void** p, uint64_t need, uint64_t& cap) {
        if (need <= cap) return true;
        const uint64_t want = std::max<uint64_t>(need, cap * 2);
        cudaFree(*p);
        *p = nullptr;
        cap = 0;
        if (cudaMalloc(p, want) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        cap = want;
        return true;
    };
    if (!grow((void**)&b->d_comp, comp_len, b->comp_cap) || !grow((void**)&b->d_out, out_len, b->out_cap) ||
        !grow((void**)&b->d_m, (uint64_t)n * sizeof(BgzfMember), b->m_cap) ||
        !grow((void**)&b->d_status, 4ull * n, b->status_cap)) {
        rc = FAME_ERR_NOMEM;
    } else {
        b->status.resize(n);
        if (cudaMemcpyAsync(b->d_comp, comp, comp_len, cudaMemcpyHostToDevice, b->st) != cudaSuccess ||
            cudaMemcpyAsync(b->d_m, m, (uint64_t)n * sizeof(BgzfMember), cudaMemcpyHostToDevice, b->st) != cudaSuccess)
            rc = FAME_ERR_CUDA;
        if (!rc) {
            k_bgzf_inflate<<<(n + BGZF_WARPS - 1) / BGZF_WARPS, 32 * BGZF_WARPS, 0, b->st>>>(b->d_comp, b->d_m, n,
                                                                                          b->d_out, b->d_status);
            if (cudaGetLastError() != cudaSuccess) rc = FAME_ERR_CUDA;
        }
        if (!rc && (cudaMemcpyAsync(b->status.data(), b->d_status, 4ull * n, cudaMemcpyDeviceToHost, b->st) != cudaSuccess ||
                    (out_len && cudaMemcpyAsync(out, b->d_out, out_len, cudaMemcpyDeviceToHost, b->st) != cudaSuccess) ||
                    cudaStreamSynchronize(b->st) != cudaSuccess))
            rc = FAME_ERR_CUDA;
        if (!rc)
            for (uint32_t i = 0; i < n; ++i)
                if (b->status[i] != INFL_OK) { rc = FAME_ERR_IO; break; }
    }
    cudaSetDevice(prev);
    return rc;
}

}  // namespace fame
