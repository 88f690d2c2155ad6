// Proof codec: the BitZ host proof stream (src/proof_codec.rs) and flock's
// LigeritoProof as a bincode 1.3 blob (src/binary_pcs.rs:487-557).
//
// Stream: lengths and small integers are u64 LE, field elements two u64 LE
// words (lo, hi), raw bytes unframed.  The Ligerito proof is embedded as
// len(u64) || blob, the blob being bincode 1.3 with fixed-width integers of
// the serde-derived LigeritoProof (flock-core/src/pcs/ligerito.rs:1509-1551):
// struct fields in declaration order without tags, Vec<T> = u64 length then
// the items, [u8; 32] = 32 raw bytes, Gf128 {lo, hi} = 16 bytes,
// SumcheckMessage {u_0, u_2} = 32 bytes.  Decoding is bounded by the blob
// length and rejects trailing bytes, like the reference's
// DefaultOptions::with_fixint_encoding().with_limit(n).reject_trailing_bytes().
#include <string.h>

#include <new>
#include <vector>

#include "../../include/bitz_gpu.h"
#include "proof.h"

namespace {

using bzp::Level;
using bzp::Rows;

constexpr uint64_t kMaxProofBytes = 64ull << 20;  // binary_pcs.rs:63

void put_u64(std::vector<uint8_t> &o, uint64_t v) {
    for (int i = 0; i < 8; ++i) o.push_back((uint8_t)(v >> (8 * i)));
}

void put_words(std::vector<uint8_t> &o, const uint64_t *w, size_t n) {
    const size_t base = o.size();
    o.resize(base + 8 * n);
    uint8_t *d = o.data() + base;
    for (size_t i = 0; i < n; ++i)
        for (int b = 0; b < 8; ++b) d[8 * i + b] = (uint8_t)(w[i] >> (8 * b));
}

void put_rows(std::vector<uint8_t> &o, const bz_rows_view &r) {
    put_u64(o, r.n_rows);
    size_t off = 0;
    for (size_t i = 0; i < r.n_rows; ++i) {
        put_u64(o, r.row_lens[i]);
        put_words(o, r.data + 2 * off, 2 * r.row_lens[i]);
        off += r.row_lens[i];
    }
}

void put_hashes(std::vector<uint8_t> &o, size_t n, const uint8_t *h) {
    put_u64(o, n);
    o.insert(o.end(), h, h + 32 * n);
}

bool rows_ok(const bz_rows_view &r) {
    if (r.n_rows && !r.row_lens) return false;
    size_t total = 0;
    for (size_t i = 0; i < r.n_rows; ++i) total += r.row_lens[i];
    return total == 0 || r.data;
}

// Bounded cursor over the blob (bincode's limit = the blob length).
struct Cursor {
    const uint8_t *p;
    size_t n, cur = 0;
    bool u64(uint64_t &v) {
        if (n - cur < 8) return false;
        v = 0;
        for (int i = 0; i < 8; ++i) v |= (uint64_t)p[cur + i] << (8 * i);
        cur += 8;
        return true;
    }
    bool bytes(uint8_t *out, size_t k) {
        if (n - cur < k) return false;
        memcpy(out, p + cur, k);
        cur += k;
        return true;
    }
    // a Vec length whose items of `item` bytes must still fit in the blob
    bool count(uint64_t &c, size_t item) {
        if (!u64(c)) return false;
        return item == 0 || c <= (n - cur) / item;
    }
    // n_words little-endian words appended to out (one geometric resize per
    // call: appending row after row stays linear in the blob size)
    template <class Vec>
    bool words(Vec &out, uint64_t n_words) {
        if ((n - cur) / 8 < n_words) return false;
        const size_t base = out.size();
        out.resize(base + n_words);
        const uint8_t *q = p + cur;
        for (uint64_t i = 0; i < n_words; ++i) {
            uint64_t w = 0;
            for (int b = 0; b < 8; ++b) w |= (uint64_t)q[8 * i + b] << (8 * b);
            out[base + i] = w;
        }
        cur += 8 * n_words;
        return true;
    }
};

bool get_rows(Cursor &c, Rows &r) {
    uint64_t n;
    if (!c.count(n, 8)) return false;
    r.lens.reserve(n);
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t len;
        if (!c.count(len, 16)) return false;
        r.lens.push_back(len);
        if (!c.words(r.data, 2 * len)) return false;
    }
    return true;
}

bool get_hashes(Cursor &c, std::vector<uint8_t> &h) {
    uint64_t n;
    if (!c.count(n, 32)) return false;
    h.resize(32 * n);
    return c.bytes(h.data(), 32 * n);
}

bool get_words_vec(Cursor &c, std::vector<uint64_t> &v, size_t words_per_item) {
    uint64_t n;
    if (!c.count(n, 8 * words_per_item)) return false;
    return c.words(v, n * words_per_item);
}

bz_rows_view rows_view(const Rows &r) {
    bz_rows_view v;
    v.n_rows = r.lens.size();
    v.row_lens = r.lens.data();
    v.data = r.data.data();
    return v;
}

}  // namespace

struct bz_writer {
    std::vector<uint8_t> buf;
};

struct bz_reader {
    const uint8_t *buf;
    size_t len, cur;
};

namespace {

int encode_blob(const bz_ligerito_proof_view *v, std::vector<uint8_t> &o) {
    if (!v || !rows_ok(v->initial_proof.rows) || !rows_ok(v->final_rows.rows))
        return BZ_ERR_ARG;
    if ((v->n_recursive_roots && !v->recursive_roots) ||
        (v->n_recursive_proofs && !v->recursive_proofs) || (v->n_yr && !v->yr) ||
        (v->n_sumcheck && !v->sumcheck) || (v->n_grinding_nonces && !v->grinding_nonces) ||
        (v->n_ood_values && !v->ood_values) ||
        (v->n_fold_grinding_nonces && !v->fold_grinding_nonces))
        return BZ_ERR_ARG;
    for (size_t i = 0; i < v->n_recursive_proofs; ++i)
        if (!rows_ok(v->recursive_proofs[i].rows)) return BZ_ERR_ARG;
    o.insert(o.end(), v->initial_root, v->initial_root + 32);
    put_rows(o, v->initial_proof.rows);
    put_hashes(o, v->initial_proof.n_hashes, v->initial_proof.hashes);
    put_hashes(o, v->n_recursive_roots, v->recursive_roots);
    put_u64(o, v->n_recursive_proofs);
    for (size_t i = 0; i < v->n_recursive_proofs; ++i) {
        put_rows(o, v->recursive_proofs[i].rows);
        put_hashes(o, v->recursive_proofs[i].n_hashes, v->recursive_proofs[i].hashes);
    }
    put_u64(o, v->n_yr);
    put_words(o, v->yr, 2 * v->n_yr);
    put_rows(o, v->final_rows.rows);
    put_hashes(o, v->final_rows.n_hashes, v->final_rows.hashes);
    put_u64(o, v->n_sumcheck);
    put_words(o, v->sumcheck, 4 * v->n_sumcheck);
    put_u64(o, v->n_grinding_nonces);
    put_words(o, v->grinding_nonces, v->n_grinding_nonces);
    put_u64(o, v->n_ood_values);
    put_words(o, v->ood_values, 2 * v->n_ood_values);
    put_u64(o, v->n_fold_grinding_nonces);
    put_words(o, v->fold_grinding_nonces, v->n_fold_grinding_nonces);
    return BZ_OK;
}

int decode_blob(const uint8_t *blob, size_t len, bz_ligerito_proof **out) {
    bz_ligerito_proof *p = new (std::nothrow) bz_ligerito_proof();
    if (!p) return BZ_ERR_NOMEM;
    Cursor c{blob, len};
    uint64_t n_rec = 0;
    bool ok = c.bytes(p->initial_root, 32) && get_rows(c, p->initial.rows) &&
              get_hashes(c, p->initial.hashes) && get_hashes(c, p->recursive_roots) &&
              c.count(n_rec, 16);  // a RecursiveProof is at least two u64 lengths
    for (uint64_t i = 0; ok && i < n_rec; ++i) {
        p->recursive.emplace_back();
        ok = get_rows(c, p->recursive.back().rows) && get_hashes(c, p->recursive.back().hashes);
    }
    ok = ok && get_words_vec(c, p->yr, 2) && get_rows(c, p->fin.rows) &&
         get_hashes(c, p->fin.hashes) && get_words_vec(c, p->sumcheck, 4) &&
         get_words_vec(c, p->grinding_nonces, 1) && get_words_vec(c, p->ood_values, 2) &&
         get_words_vec(c, p->fold_grinding_nonces, 1);
    if (!ok || c.cur != len) {  // truncated / oversized lengths / trailing bytes
        delete p;
        return BZ_ERR_DECODE;
    }
    *out = p;
    return BZ_OK;
}

}  // namespace

extern "C" {

int bz_ligerito_proof_encode(const bz_ligerito_proof_view *view, uint8_t *out, size_t cap,
                             size_t *len) {
    if (!len) return BZ_ERR_ARG;
    if (!out) {  // size query: the byte count follows from the view's lengths
        if (!view || !rows_ok(view->initial_proof.rows) || !rows_ok(view->final_rows.rows) ||
            (view->n_recursive_proofs && !view->recursive_proofs))
            return BZ_ERR_ARG;
        for (size_t i = 0; i < view->n_recursive_proofs; ++i)
            if (!rows_ok(view->recursive_proofs[i].rows)) return BZ_ERR_ARG;
        auto rows_bytes = [](const bz_rows_view &r) {
            size_t b = 8;
            for (size_t i = 0; i < r.n_rows; ++i) b += 8 + 16 * (size_t)r.row_lens[i];
            return b;
        };
        size_t n = 32 + rows_bytes(view->initial_proof.rows) + 8 + 32 * view->initial_proof.n_hashes +
                   8 + 32 * view->n_recursive_roots + 8;
        for (size_t i = 0; i < view->n_recursive_proofs; ++i)
            n += rows_bytes(view->recursive_proofs[i].rows) + 8 +
                 32 * view->recursive_proofs[i].n_hashes;
        n += 8 + 16 * view->n_yr + rows_bytes(view->final_rows.rows) + 8 +
             32 * view->final_rows.n_hashes + 8 + 32 * view->n_sumcheck + 8 +
             8 * view->n_grinding_nonces + 8 + 16 * view->n_ood_values + 8 +
             8 * view->n_fold_grinding_nonces;
        *len = n;
        return BZ_OK;
    }
    std::vector<uint8_t> o;
    int rc = encode_blob(view, o);
    if (rc) return rc;
    *len = o.size();
    if (!out) return BZ_OK;
    if (cap < o.size()) return BZ_ERR_ARG;
    memcpy(out, o.data(), o.size());
    return BZ_OK;
}

int bz_ligerito_proof_decode(const uint8_t *blob, size_t len, bz_ligerito_proof **out) {
    if (!out || (len && !blob)) return BZ_ERR_ARG;
    *out = nullptr;
    return decode_blob(blob, len, out);
}

int bz_ligerito_proof_view_of(bz_ligerito_proof *p, bz_ligerito_proof_view *v) {
    if (!p || !v) return BZ_ERR_ARG;
    p->recursive_views.clear();
    for (const Level &l : p->recursive) {
        bz_level_view lv;
        lv.rows = rows_view(l.rows);
        lv.n_hashes = l.hashes.size() / 32;
        lv.hashes = l.hashes.data();
        p->recursive_views.push_back(lv);
    }
    memcpy(v->initial_root, p->initial_root, 32);
    v->initial_proof.rows = rows_view(p->initial.rows);
    v->initial_proof.n_hashes = p->initial.hashes.size() / 32;
    v->initial_proof.hashes = p->initial.hashes.data();
    v->n_recursive_roots = p->recursive_roots.size() / 32;
    v->recursive_roots = p->recursive_roots.data();
    v->n_recursive_proofs = p->recursive_views.size();
    v->recursive_proofs = p->recursive_views.data();
    v->n_yr = p->yr.size() / 2;
    v->yr = p->yr.data();
    v->final_rows.rows = rows_view(p->fin.rows);
    v->final_rows.n_hashes = p->fin.hashes.size() / 32;
    v->final_rows.hashes = p->fin.hashes.data();
    v->n_sumcheck = p->sumcheck.size() / 4;
    v->sumcheck = p->sumcheck.data();
    v->n_grinding_nonces = p->grinding_nonces.size();
    v->grinding_nonces = p->grinding_nonces.data();
    v->n_ood_values = p->ood_values.size() / 2;
    v->ood_values = p->ood_values.data();
    v->n_fold_grinding_nonces = p->fold_grinding_nonces.size();
    v->fold_grinding_nonces = p->fold_grinding_nonces.data();
    return BZ_OK;
}

int bz_ligerito_proof_free(bz_ligerito_proof *p) {
    delete p;
    return BZ_OK;
}

// ---- stream writer / reader (src/proof_codec.rs:39-161) ----------------------

int bz_writer_create(bz_writer **out) {
    if (!out) return BZ_ERR_ARG;
    *out = new (std::nothrow) bz_writer();
    return *out ? BZ_OK : BZ_ERR_NOMEM;
}

int bz_writer_destroy(bz_writer *w) {
    delete w;
    return BZ_OK;
}

int bz_writer_len(bz_writer *w, uint64_t n) {
    if (!w) return BZ_ERR_ARG;
    put_u64(w->buf, n);
    return BZ_OK;
}

int bz_writer_gf(bz_writer *w, const uint64_t g[2]) {
    if (!w || !g) return BZ_ERR_ARG;
    put_words(w->buf, g, 2);
    return BZ_OK;
}

int bz_writer_bytes(bz_writer *w, const uint8_t *data, size_t len) {
    if (!w || (len && !data)) return BZ_ERR_ARG;
    w->buf.insert(w->buf.end(), data, data + len);
    return BZ_OK;
}

int bz_writer_data(const bz_writer *w, const uint8_t **data, size_t *len) {
    if (!w || !data || !len) return BZ_ERR_ARG;
    *data = w->buf.data();
    *len = w->buf.size();
    return BZ_OK;
}

int bz_write_round0(bz_writer *w, const uint64_t y[2], int has_nonce, uint64_t nonce) {
    if (!w || !y) return BZ_ERR_ARG;
    put_words(w->buf, y, 2);
    put_u64(w->buf, has_nonce ? 1 : 0);
    if (has_nonce) put_u64(w->buf, nonce);
    return BZ_OK;
}

int bz_write_ring_switch(bz_writer *w, const uint64_t s_v[256]) {
    if (!w || !s_v) return BZ_ERR_ARG;
    put_words(w->buf, s_v, 256);
    return BZ_OK;
}

int bz_write_ligerito(bz_writer *w, const bz_ligerito_proof_view *view) {
    if (!w) return BZ_ERR_ARG;
    std::vector<uint8_t> blob;
    int rc = encode_blob(view, blob);
    if (rc) return rc;
    put_u64(w->buf, blob.size());
    w->buf.insert(w->buf.end(), blob.begin(), blob.end());
    return BZ_OK;
}

int bz_reader_create(const uint8_t *buf, size_t len, bz_reader **out) {
    if (!out || (len && !buf)) return BZ_ERR_ARG;
    *out = new (std::nothrow) bz_reader{buf, len, 0};
    return *out ? BZ_OK : BZ_ERR_NOMEM;
}

int bz_reader_destroy(bz_reader *r) {
    delete r;
    return BZ_OK;
}

size_t bz_reader_remaining(const bz_reader *r) { return r ? r->len - r->cur : 0; }

int bz_reader_len(bz_reader *r, uint64_t *n) {
    if (!r || !n) return BZ_ERR_ARG;
    if (r->len - r->cur < 8) return BZ_ERR_TRUNCATED;
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)r->buf[r->cur + i] << (8 * i);
    r->cur += 8;
    *n = v;
    return BZ_OK;
}

int bz_reader_gf(bz_reader *r, uint64_t g[2]) {
    if (!r || !g) return BZ_ERR_ARG;
    if (r->len - r->cur < 16) return BZ_ERR_TRUNCATED;
    bz_reader_len(r, &g[0]);
    bz_reader_len(r, &g[1]);
    return BZ_OK;
}

int bz_reader_take(bz_reader *r, size_t n, const uint8_t **data) {
    if (!r || !data) return BZ_ERR_ARG;
    if (r->len - r->cur < n) return BZ_ERR_TRUNCATED;
    *data = r->buf + r->cur;
    r->cur += n;
    return BZ_OK;
}

int bz_read_round0(bz_reader *r, uint64_t y[2], int *has_nonce, uint64_t *nonce) {
    if (!r || !y || !has_nonce || !nonce) return BZ_ERR_ARG;
    int rc = bz_reader_gf(r, y);
    if (rc) return rc;
    uint64_t tag;
    rc = bz_reader_len(r, &tag);
    if (rc) return rc;
    if (tag > 1) return BZ_ERR_NONCANONICAL;
    *has_nonce = (int)tag;
    *nonce = 0;
    return tag ? bz_reader_len(r, nonce) : BZ_OK;
}

int bz_read_ring_switch(bz_reader *r, uint64_t s_v[256]) {
    if (!r || !s_v) return BZ_ERR_ARG;
    if (r->len - r->cur < 128 * 16) return BZ_ERR_TRUNCATED;
    for (int i = 0; i < 128; ++i) bz_reader_gf(r, s_v + 2 * i);
    return BZ_OK;
}

int bz_read_ligerito(bz_reader *r, bz_ligerito_proof **out) {
    if (!r || !out) return BZ_ERR_ARG;
    *out = nullptr;
    uint64_t n;
    int rc = bz_reader_len(r, &n);
    if (rc) return rc;
    if (n > kMaxProofBytes || n > r->len - r->cur) return BZ_ERR_TRUNCATED;
    rc = decode_blob(r->buf + r->cur, (size_t)n, out);
    if (rc) return rc;
    r->cur += (size_t)n;
    return BZ_OK;
}

}  // extern "C"
