"""Host-side mirror of the reference's commit / open interface, backed by the
GB300 library.

Names, argument meaning and error behaviour follow flock-core's
``pcs::commit`` (``PcsParams``, ``commit``, ``Commitment``, ``ProverData``),
``pcs::ligerito::ligero_commit`` and ``merkle::merkle_multi_proof``, and the
``SumcheckProver`` fold of ``pcs::ligerito`` (paths relative to
vendor/flock-mod/crates/flock-core/src in BitZ-PoC).  Shape violations that the
reference ``assert!``s raise ``ValueError`` here; device failures raise
``BzError``.
"""
from __future__ import annotations

import atexit
import ctypes
import threading
import weakref
from dataclasses import dataclass

import numpy as np

from ._lib import BzError, Params, check, lib, ptr

LOG_PACKING = 7  # flock-core/src/pcs/pack.rs (128 bits per GF(2^128) word)


class HashKind:
    """flock-core/src/hash.rs:21-27 (SHA-256 is the crate default)."""
    SHA256 = 0
    BLAKE3 = 1


@dataclass
class PcsParams:
    """flock-core/src/pcs/commit.rs:31-137."""
    m: int
    log_inv_rate: int
    log_batch_size: int = 5
    merkle_hash: int = HashKind.SHA256

    def log_msg_len(self) -> int:
        return self.m - LOG_PACKING

    def log_dim(self) -> int:
        return self.log_msg_len() - self.log_batch_size

    def k_code(self) -> int:
        return self.log_dim() + self.log_inv_rate

    def n_positions(self) -> int:
        return 1 << self.k_code()

    def num_ntts(self) -> int:
        return 1 << self.log_batch_size

    def codeword_len_f128(self) -> int:
        return self.n_positions() * self.num_ntts()

    def n_leaves(self) -> int:
        return self.codeword_len_f128() >> self.log_batch_size

    def leaf_size_bytes(self) -> int:
        return 16 << self.log_batch_size

    def validate(self):
        # commit.rs:125-136
        if self.m < LOG_PACKING + self.log_batch_size:
            raise ValueError(
                f"m={self.m} too small (need m >= LOG_PACKING + log_batch_size = "
                f"{LOG_PACKING + self.log_batch_size})")
        if self.log_inv_rate < 1:
            raise ValueError("log_inv_rate must be >= 1 for a non-trivial RS code")

    def to_c(self) -> Params:
        return Params(self.log_msg_len(), self.log_inv_rate, self.log_batch_size, self.merkle_hash)


_contexts: "weakref.WeakSet[Context]" = weakref.WeakSet()


class Context:
    """One device context (stream, memory budget, twiddle and schedule caches).

    Objects that hold device resources of this context (device arrays,
    commitments, openings, batch plans, servers) register with it; ``close``
    releases them first, then the context, and every open context is closed
    at interpreter exit, so teardown order never depends on the garbage
    collector."""

    def __init__(self, device: int = 0, mem_budget_bytes: int = 0):
        L = lib()
        h = ctypes.c_void_p()
        check(None, L.bz_ctx_create(device, mem_budget_bytes, ctypes.byref(h)))
        self.handle = h
        self.device = device
        self._children = weakref.WeakSet()
        _contexts.add(self)

    def adopt(self, obj):
        """Register obj (with a ``release()`` method) for release before close."""
        self._children.add(obj)
        return obj

    def close(self):
        if self.handle:
            for ch in list(self._children):
                try:
                    ch.release()
                except Exception:
                    pass
            lib().bz_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib().bz_ctx_stream(self.handle) or 0

    def synchronize(self):
        check(self.handle, lib().bz_ctx_synchronize(self.handle))

    def memory(self):
        used, budget = ctypes.c_uint64(), ctypes.c_uint64()
        check(self.handle, lib().bz_ctx_memory(self.handle, ctypes.byref(used), ctypes.byref(budget)))
        return used.value, budget.value

    def kernel_launches(self) -> int:
        return int(lib().bz_kernel_launches(self.handle))

    def timer_begin(self):
        check(self.handle, lib().bz_timer_begin(self.handle))

    def timer_end(self) -> float:
        ms = ctypes.c_float()
        check(self.handle, lib().bz_timer_end(self.handle, ctypes.byref(ms)))
        return ms.value

    def commit_profile(self, msg: "DeviceArray", params: PcsParams):
        """[(kernel name, ms)] for one commit, one entry per launch."""
        p = params.to_c()
        cap = 256
        ms = np.zeros(cap, np.float32)
        names = ctypes.create_string_buffer(cap * 32)
        n = ctypes.c_size_t()
        root = (ctypes.c_uint8 * 32)()
        check(self.handle, lib().bz_commit_profile(self.handle, msg.ptr, msg.n, ctypes.byref(p),
                                                   cap, ptr(ms), names, ctypes.byref(n), root))
        out = []
        for i in range(min(n.value, cap)):
            nm = names.raw[32 * i:32 * i + 32].split(b"\0")[0].decode()
            out.append((nm, float(ms[i])))
        return out, bytes(root)

    def autotune(self, params: PcsParams, reps: int = 3) -> int:
        p = params.to_c()
        out = ctypes.c_uint32()
        check(self.handle, lib().bz_autotune(self.handle, ctypes.byref(p), reps, ctypes.byref(out)))
        return out.value

    def schedule(self, params: PcsParams) -> int:
        p = params.to_c()
        out = ctypes.c_uint32()
        check(self.handle, lib().bz_schedule_get(self.handle, ctypes.byref(p), ctypes.byref(out)))
        return out.value

    def set_schedule(self, params: PcsParams, schedule: int):
        p = params.to_c()
        check(self.handle, lib().bz_schedule_set(self.handle, ctypes.byref(p), schedule))


_default = None
_default_lock = threading.Lock()


@atexit.register
def _close_contexts():
    for c in list(_contexts):
        c.close()


def default_context() -> Context:
    global _default
    with _default_lock:
        if _default is None:
            _default = Context(0)
        return _default


class DeviceArray:
    """GF(2^128) elements in device memory ((n, 2) uint64 on the host side)."""

    def __init__(self, n: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.n = int(n)
        p = ctypes.c_void_p()
        check(self.ctx.handle, lib().bz_device_alloc(self.ctx.handle, max(self.n, 1) * 16,
                                                     ctypes.byref(p)))
        self.ptr = p
        self.ctx.adopt(self)

    @classmethod
    def from_host(cls, a: np.ndarray, ctx: Context | None = None) -> "DeviceArray":
        a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2)
        d = cls(a.shape[0], ctx)
        check(d.ctx.handle, lib().bz_memcpy_h2d(d.ctx.handle, d.ptr, ptr(a), a.nbytes))
        return d

    @classmethod
    def chacha(cls, seed: int, n: int, ctx: Context | None = None) -> "DeviceArray":
        d = cls(n, ctx)
        check(d.ctx.handle, lib().bz_chacha_fill_device(d.ctx.handle, seed, 0, d.ptr, n))
        return d

    def to_host(self) -> np.ndarray:
        out = np.zeros((self.n, 2), np.uint64)
        check(self.ctx.handle, lib().bz_memcpy_d2h(self.ctx.handle, ptr(out), self.ptr, out.nbytes))
        return out

    def free(self):
        if self.ptr:
            if self.ctx.handle:  # a closed context already released its memory
                lib().bz_device_free(self.ctx.handle, self.ptr)
            self.ptr = None

    release = free

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


@dataclass
class Commitment:
    """commit.rs:140-145: Merkle root + params."""
    root: bytes
    params: PcsParams


class ProverData:
    """commit.rs:146-163, kept on the device: the codeword and Merkle tree
    stay resident until ``free`` (the reference recycles them on Drop)."""

    def __init__(self, handle, params: PcsParams, ctx: Context):
        self.handle = handle
        self.params = params
        self.ctx = ctx
        ctx.adopt(self)

    def _h(self):
        if not self.handle:
            raise BzError(7, "prover data already freed")
        return self.handle

    @property
    def codeword(self) -> np.ndarray:
        n = self.params.codeword_len_f128()
        out = np.zeros((n, 2), np.uint64)
        check(self.ctx.handle, lib().bz_commitment_copy_codeword(self._h(), ptr(out), n))
        return out

    @property
    def merkle_tree(self) -> np.ndarray:
        n = 2 * self.params.n_leaves() - 1
        out = np.zeros((n, 32), np.uint8)
        check(self.ctx.handle, lib().bz_commitment_copy_tree(self._h(), ptr(out), n))
        return out

    def device_ptrs(self):
        cw, tr = ctypes.c_void_p(), ctypes.c_void_p()
        check(self.ctx.handle, lib().bz_commitment_device_ptrs(self._h(), ctypes.byref(cw),
                                                               ctypes.byref(tr)))
        return cw.value, tr.value

    def rows(self, positions) -> np.ndarray:
        """Opened rows (ligerito.rs:3476-3479): shape (q, lanes, 2)."""
        pos = np.ascontiguousarray(np.asarray(positions, dtype=np.uint64))
        out = np.zeros((len(pos), self.params.num_ntts(), 2), np.uint64)
        check(self.ctx.handle, lib().bz_commitment_rows(self._h(), ptr(pos) if len(pos) else None,
                                                        len(pos), ptr(out)))
        return out

    def multi_proof(self, positions) -> np.ndarray:
        """merkle_multi_proof (merkle.rs:688-741) against this tree."""
        pos = np.ascontiguousarray(np.asarray(positions, dtype=np.uint64))
        n = ctypes.c_size_t()
        L = lib()
        pp = ptr(pos) if len(pos) else None
        check(self.ctx.handle, L.bz_commitment_multiproof(self._h(), pp, len(pos), None, 0,
                                                          ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), 32), np.uint8)
        check(self.ctx.handle, L.bz_commitment_multiproof(self._h(), pp, len(pos), ptr(out),
                                                          n.value, ctypes.byref(n)))
        return out[:n.value]

    def free(self):
        if self.handle:
            if self.ctx.handle:  # a closed context already freed its commitments
                lib().bz_commitment_free(self.handle)
            self.handle = None

    release = free

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _to_commit(handle, params, ctx, root_buf):
    return Commitment(bytes(root_buf), params), ProverData(handle, params, ctx)


def commit(z_packed, params: PcsParams, ctx: Context | None = None):
    """flock_core::pcs::commit::commit (commit.rs:180-200).

    ``z_packed``: host array of 2^(m-7) elements ((n, 2) uint64) or a
    ``DeviceArray``.  Returns ``(Commitment, ProverData)``.
    """
    ctx = ctx or default_context()
    params.validate()
    p = params.to_c()
    h = ctypes.c_void_p()
    root = (ctypes.c_uint8 * 32)()
    L = lib()
    if isinstance(z_packed, DeviceArray):
        n = z_packed.n
        if n != 1 << params.log_msg_len():
            raise ValueError("z_packed.len() must equal 2^(m - 7)")
        check(ctx.handle, L.bz_commit_device(ctx.handle, z_packed.ptr, n, ctypes.byref(p),
                                             ctypes.byref(h), root))
    else:
        a = np.ascontiguousarray(z_packed, dtype=np.uint64).reshape(-1, 2)
        if a.shape[0] != 1 << params.log_msg_len():
            raise ValueError("z_packed.len() must equal 2^(m - 7)")
        check(ctx.handle, L.bz_commit(ctx.handle, ptr(a), a.shape[0], ctypes.byref(p),
                                      ctypes.byref(h), root))
    return _to_commit(h, params, ctx, root)


@dataclass
class LigeroWitness:
    """ligerito.rs:2355-2378: codeword matrix + tree, device resident."""
    data: ProverData
    block_len: int
    num_interleaved: int
    root: bytes


def ligero_commit(poly, log_msg_cols: int, log_num_interleaved: int, log_inv_rate: int,
                  kind: int = HashKind.SHA256, ctx: Context | None = None) -> LigeroWitness:
    """ligerito.rs:2390-2434 (poly[col * num_interleaved + lane])."""
    ctx = ctx or default_context()
    dev = poly if isinstance(poly, DeviceArray) else DeviceArray.from_host(poly, ctx)
    if dev.n != 1 << (log_msg_cols + log_num_interleaved):
        raise ValueError("poly.len() must equal num_interleaved * msg_cols")
    h = ctypes.c_void_p()
    root = (ctypes.c_uint8 * 32)()
    check(ctx.handle, lib().bz_ligero_commit_device(ctx.handle, dev.ptr, log_msg_cols,
                                                    log_num_interleaved, log_inv_rate, kind,
                                                    ctypes.byref(h), root))
    params = PcsParams(log_msg_cols + log_num_interleaved + LOG_PACKING, log_inv_rate,
                       log_num_interleaved, kind)
    return LigeroWitness(ProverData(h, params, ctx), (1 << log_msg_cols) << log_inv_rate,
                         1 << log_num_interleaved, bytes(root))


def commit_batch(msgs, params_list, use_graph: bool = True, ctx: Context | None = None):
    """Many independent commits in one CUDA-graph launch (device messages)."""
    ctx = ctx or default_context()
    n = len(msgs)
    arr = (ctypes.c_void_p * n)(*[m.ptr.value if hasattr(m.ptr, "value") else m.ptr for m in msgs])
    ps = (Params * n)(*[p.to_c() for p in params_list])
    outs = (ctypes.c_void_p * n)()
    roots = np.zeros((n, 32), np.uint8)
    check(ctx.handle, lib().bz_commit_batch_device(ctx.handle, n, arr, ps, outs, ptr(roots),
                                                   1 if use_graph else 0))
    res = []
    for i in range(n):
        res.append((Commitment(roots[i].tobytes(), params_list[i]),
                    ProverData(ctypes.c_void_p(outs[i]), params_list[i], ctx)))
    return res


def chacha_words(seed: int, n: int, first_word: int = 0, n_threads: int = 0) -> np.ndarray:
    """Synthetic inputs: RFC 8439 ChaCha20 words (host)."""
    import os

    out = np.zeros((n, 2), np.uint64)
    check(None, lib().bz_chacha_fill_host(seed, first_word, ptr(out), n,
                                          n_threads or (os.cpu_count() or 1)))
    return out


class BatchPlan:
    """Reusable batched commit (bz_batch_plan_*): resident buffers for every
    polynomial and, with ``use_graph``, one CUDA graph holding all kernels,
    spread over ``n_branches`` parallel branches.  With ``persistent`` every
    commit runs as work items of one persistent kernel
    (bz_batch_plan_create_persistent), launched through a CUDA graph."""

    def __init__(self, msgs, params_list, use_graph: bool = True, n_branches: int = 4,
                 ctx: Context | None = None, persistent: bool = False):
        self.ctx = ctx or default_context()
        L = lib()
        for name, res, args in (
                ("bz_batch_plan_create", ctypes.c_int,
                 [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.POINTER(Params),
                  ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
                ("bz_batch_plan_create_persistent", ctypes.c_int,
                 [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.POINTER(Params),
                  ctypes.POINTER(ctypes.c_void_p)]),
                ("bz_batch_plan_launch", ctypes.c_int, [ctypes.c_void_p]),
                ("bz_batch_plan_roots", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
                ("bz_batch_plan_commitment", ctypes.c_void_p, [ctypes.c_void_p, ctypes.c_size_t]),
                ("bz_batch_plan_destroy", ctypes.c_int, [ctypes.c_void_p])):
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        self.L = L
        self.n = len(msgs)
        self.params = list(params_list)
        self._msgs = msgs
        arr = (ctypes.c_void_p * self.n)(*[m.ptr.value if hasattr(m.ptr, "value") else m.ptr
                                           for m in msgs])
        ps = (Params * self.n)(*[p.to_c() for p in self.params])
        h = ctypes.c_void_p()
        if persistent:
            check(self.ctx.handle, L.bz_batch_plan_create_persistent(
                self.ctx.handle, self.n, arr, ps, ctypes.byref(h)))
        else:
            check(self.ctx.handle, L.bz_batch_plan_create(self.ctx.handle, self.n, arr, ps,
                                                          1 if use_graph else 0, n_branches,
                                                          ctypes.byref(h)))
        self.h = h
        self.ctx.adopt(self)

    def launch(self):
        check(self.ctx.handle, self.L.bz_batch_plan_launch(self.h))

    def roots(self) -> list[bytes]:
        out = np.zeros((self.n, 32), np.uint8)
        check(self.ctx.handle, self.L.bz_batch_plan_roots(self.h, ptr(out)))
        return [out[i].tobytes() for i in range(self.n)]

    def codeword(self, i: int) -> np.ndarray:
        c = self.L.bz_batch_plan_commitment(self.h, i)
        n = self.params[i].codeword_len_f128()
        out = np.zeros((n, 2), np.uint64)
        check(self.ctx.handle, lib().bz_commitment_copy_codeword(c, ptr(out), n))
        return out

    def close(self):
        if self.h:
            if self.ctx.handle:
                self.L.bz_batch_plan_destroy(self.h)
            self.h = None

    release = close

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
