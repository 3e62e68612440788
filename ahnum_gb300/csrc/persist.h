// Checkpoint files, byte-compatible with the reference's:
//   Fermat  "KITECKP1" (also reads the legacy "AHNCKPT1"): header {magic[8], k, n, base, iter,
//           nlimbs, fft_len} as u64s, x limbs, d limbs, FNV-1a 64 of all of it (src/prp.c:146-212)
//   LLR     "KITELLR1": header {magic[8], k, n, P, iter, nlimbs, fft_len, run, prev[2]}, x limbs,
//           FNV-1a 64 (src/llr.c:92-146)
// Files are written to "<path>.tmp" and renamed over the old one.
#pragma once

#include <cstdint>
#include <vector>

namespace kg {

struct PrpCheckpointHeader {
    char magic[8];
    uint64_t k, n, base, iter, nlimbs, fft_len;
};

struct LlrCheckpointHeader {
    char magic[8];
    uint64_t k, n, P, iter, nlimbs, fft_len, run;
    uint64_t prev[2];
};

bool prp_checkpoint_write(const char *path, uint64_t k, uint64_t n, uint32_t base, uint64_t iter,
                          uint32_t fft_len, const std::vector<uint64_t> &x, const std::vector<uint64_t> &d);
bool prp_checkpoint_read(const char *path, uint64_t k, uint64_t n, uint32_t base, size_t nlimbs,
                         uint64_t &iter, uint32_t &fft_len, std::vector<uint64_t> &x, std::vector<uint64_t> &d);
bool prp_checkpoint_header(const char *path, PrpCheckpointHeader &h);

bool llr_checkpoint_write(const char *path, const LlrCheckpointHeader &h, const std::vector<uint64_t> &x);
bool llr_checkpoint_read(const char *path, size_t nlimbs, LlrCheckpointHeader &h, std::vector<uint64_t> &x);
// The header alone (magic checked, checksum not), as the reference's kite_llr_checkpoint_iter
// reads it (src/llr.c:135-146).
bool llr_checkpoint_header(const char *path, LlrCheckpointHeader &h);

}  // namespace kg
