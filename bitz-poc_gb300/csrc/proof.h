// Host representation of flock's LigeritoProof (flock-core/src/pcs/
// ligerito.rs:1509-1551), shared by the codec (codec.cpp) and the prover
// (open.cu).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../../include/bitz_gpu.h"

namespace bzp {

struct Rows {
    std::vector<size_t> lens;
    std::vector<uint64_t> data;  // concatenated rows, 2 words per element
};

struct Level {
    Rows rows;
    std::vector<uint8_t> hashes;  // 32 bytes each
};

}  // namespace bzp

struct bz_ligerito_proof {
    uint8_t initial_root[32];
    bzp::Level initial;
    std::vector<uint8_t> recursive_roots;
    std::vector<bzp::Level> recursive;
    std::vector<bz_level_view> recursive_views;  // filled by bz_ligerito_proof_view_of
    std::vector<uint64_t> yr;
    bzp::Level fin;
    std::vector<uint64_t> sumcheck;  // 4 words per message
    std::vector<uint64_t> grinding_nonces;
    std::vector<uint64_t> ood_values;
    std::vector<uint64_t> fold_grinding_nonces;
};
