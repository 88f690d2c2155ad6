// Host representation of flock's LigeritoProof (flock-core/src/pcs/
// ligerito.rs:1509-1551), shared by the codec (codec.cpp) and the prover
// (open.cu).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <memory>
#include <new>
#include <utility>
#include <vector>

#include "../../include/bitz_gpu.h"

namespace bzp {

// Allocator whose resize leaves new elements uninitialised: opened rows are
// written in full by a device copy right after the resize, so zero-filling
// megabytes first would only touch the pages twice.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U> &) {}
    template <class U>
    void construct(U *p) {
        ::new (static_cast<void *>(p)) U;
    }
    template <class U, class... Args>
    void construct(U *p, Args &&...args) {
        ::new (static_cast<void *>(p)) U(std::forward<Args>(args)...);
    }
};

struct Rows {
    std::vector<size_t> lens;
    std::vector<uint64_t, NoInitAlloc<uint64_t>> data;  // concatenated rows, 2 words each
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
