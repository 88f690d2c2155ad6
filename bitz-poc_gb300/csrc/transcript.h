// Host BLAKE3 hasher and the BitZ Blake3Transcript built on it (definitions in
// transcript.cu).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include "../../include/bitz_gpu.h"

namespace bzh {

// A compression input whose output is either a chaining value or, with the
// ROOT flag and counter t, block t of the extended output.
struct Node {
    uint32_t cv[8];
    uint32_t block[16];
    uint64_t counter;
    uint32_t block_len, flags;
    void chaining_value(uint32_t out[8]) const;
    void root_output(uint8_t *out, size_t n) const;
};

class Hasher {
  public:
    Hasher();
    void update(const uint8_t *p, size_t n);
    // finalize_xof().fill(out): does not change the state
    void xof(uint8_t *out, size_t n) const;

  private:
    void reset_chunk(uint64_t index);
    void push_chunk_cv(const uint32_t cv[8], uint64_t completed);
    Node chunk_node() const;
    Node root_node() const;
    uint32_t chunk_cv_[8];
    uint64_t chunk_index_ = 0;
    uint8_t buf_[64];
    uint32_t buf_len_ = 0, blocks_done_ = 0;
    uint32_t stack_[54][8];  // 2^54 chunks = 2^64 bytes
    int depth_ = 0;
};

struct Transcript {
    Hasher h;
    void absorb_slice(const uint8_t *p, size_t n);
    // get_challenge of an n-byte type without padding bits
    void challenge(uint8_t *out, size_t n);
    // get_field_challenge::<Gf128>: 16 squeezed bytes as two LE words
    void sample_f128(uint64_t out[2]);
    // ZincChallenger::observe_f128 (src/ligerito_flock.rs:41-46)
    void observe_f128(const uint64_t v[2]);
    void fill_sampling_bytes(uint8_t *out, size_t n);
};

}  // namespace bzh

bzh::Transcript *bz_transcript_inner(bz_transcript *t);
