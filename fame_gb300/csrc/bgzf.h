// BGZF members inflated on the GPU (library-internal interface of the FASTQ
// reader): one warp per member, the members' sizes known from their headers
// and trailers, so every member's output has its place before the launch.
#pragma once
#include <stdint.h>

namespace fame {

struct BgzfMember {
    uint64_t coff;    // raw DEFLATE stream: offset in the compressed span
    uint32_t clen;    //   and length
    uint32_t crc;     // the trailer's CRC-32 of the output
    uint64_t ooff;    // output offset
    uint32_t isize;   // output bytes (the trailer's ISIZE)
    uint32_t pad;
};

struct BgzfGpu;

// Device buffers and a stream on `device`; nullptr when the device cannot be used.
BgzfGpu* bgzf_gpu_open(int device);
void bgzf_gpu_close(BgzfGpu* b);
// Inflates the n members of comp[0 .. comp_len) (host memory) into
// out[0 .. out_len) (host memory; out_len = the members' summed ISIZE).
// FAME_OK; FAME_ERR_IO when a member's stream is malformed or its size or
// CRC-32 differs from its trailer; FAME_ERR_CUDA / FAME_ERR_NOMEM.
int bgzf_gpu_inflate(BgzfGpu* b, const uint8_t* comp, uint64_t comp_len, const BgzfMember* m, uint32_t n,
                     uint8_t* out, uint64_t out_len);

}  // namespace fame
