"""Continuous-batching commit/open server (C ABI bz_server_*).

``Server.submit_commit`` queues a commit of a host message; the native
scheduler admits it when an execution slot and device memory are free.
``submit_open`` queues the opening (rows + multi-proof) of a committed
request, after which its resident codeword and tree are freed;
``submit_commit_open`` runs both back to back on one stream.  Queued commits
are admitted smallest first (a request that waited past the aging bound goes
first), small requests on high-priority streams (``set_policy``).  ``next_done`` is the completion
queue: the ids of requests whose state changed, without polling each one.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import Params, check, lib, ptr
from .pcs import Context, PcsParams, default_context

QUEUED, RUNNING, COMMITTED, OPEN_QUEUED, OPENING, OPENED, FAILED = range(7)
ADMIT_FIFO, ADMIT_SMALLEST = 0, 1

_P = ctypes.c_void_p
_S = ctypes.c_size_t
_U64 = ctypes.c_uint64

_SIGS = {
    "bz_server_create": (ctypes.c_int, [_P, ctypes.c_int, _U64, _S, ctypes.POINTER(_P)]),
    "bz_server_submit_commit": (ctypes.c_int, [_P, _P, _S, ctypes.POINTER(Params),
                                               ctypes.POINTER(_U64)]),
    "bz_server_submit_commit_open": (ctypes.c_int, [_P, _P, _S, ctypes.POINTER(Params), _P, _S,
                                                    ctypes.POINTER(_U64)]),
    "bz_server_submit_open": (ctypes.c_int, [_P, _U64, _P, _S]),
    "bz_server_next_done": (ctypes.c_int, [_P, _P, _P, _S, ctypes.POINTER(_S), ctypes.c_uint32]),
    "bz_server_poll": (ctypes.c_int, [_P, _U64, ctypes.POINTER(ctypes.c_int)]),
    "bz_server_wait": (ctypes.c_int, [_P, _U64, ctypes.c_int, ctypes.c_uint32]),
    "bz_server_root": (ctypes.c_int, [_P, _U64, _P]),
    "bz_server_open_result": (ctypes.c_int, [_P, _U64, _P, _S, _P, _S, ctypes.POINTER(_S),
                                             ctypes.POINTER(_S)]),
    "bz_server_times": (ctypes.c_int, [_P, _U64, _P]),
    "bz_server_release": (ctypes.c_int, [_P, _U64]),
    "bz_server_stats": (ctypes.c_int, [_P] + [ctypes.POINTER(_U64)] * 5),
    "bz_server_destroy": (ctypes.c_int, [_P]),
    "bz_server_set_policy": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_uint32, ctypes.c_int]),
}


def _declare():
    L = lib()
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


class Server:
    def __init__(self, ctx: Context | None = None, n_slots: int = 4, mem_budget_bytes: int = 0,
                 queue_cap: int = 0):
        self.ctx = ctx or default_context()
        self.L = _declare()
        h = _P()
        check(self.ctx.handle, self.L.bz_server_create(self.ctx.handle, n_slots, mem_budget_bytes,
                                                       queue_cap, ctypes.byref(h)))
        self.h = h
        self._keep = {}  # request id -> host buffer kept alive until committed
        self.ctx.adopt(self)

    def close(self):
        if self.h:
            if self.ctx.handle:
                self.L.bz_server_destroy(self.h)
            self.h = None

    release = close

    def set_policy(self, admit_order: int = ADMIT_SMALLEST, aging_ms: int = 500,
                   high_priority_log_size: int = 20) -> None:
        """Admission order (smallest first with an aging bound, or arrival
        order) and the largest request (log2 elements) that runs on
        high-priority streams (-1: none)."""
        check(self.ctx.handle, self.L.bz_server_set_policy(self.h, admit_order, aging_ms,
                                                           high_priority_log_size))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit_commit(self, msg: np.ndarray, params: PcsParams) -> int:
        msg = np.ascontiguousarray(msg, dtype=np.uint64).reshape(-1, 2)
        p = params.to_c()
        rid = _U64()
        check(self.ctx.handle, self.L.bz_server_submit_commit(self.h, ptr(msg), msg.shape[0],
                                                              ctypes.byref(p), ctypes.byref(rid)))
        self._keep[rid.value] = msg
        return rid.value

    def submit_commit_ptr(self, host_ptr: int, n_words: int, params: PcsParams) -> int:
        p = params.to_c()
        rid = _U64()
        check(self.ctx.handle, self.L.bz_server_submit_commit(self.h, host_ptr, n_words,
                                                              ctypes.byref(p), ctypes.byref(rid)))
        return rid.value

    def submit_commit_open(self, msg: np.ndarray, params: PcsParams, positions) -> int:
        msg = np.ascontiguousarray(msg, dtype=np.uint64).reshape(-1, 2)
        rid = self.submit_commit_open_ptr(msg.ctypes.data, msg.shape[0], params, positions)
        self._keep[rid] = msg
        return rid

    def submit_commit_open_ptr(self, host_ptr: int, n_words: int, params: PcsParams,
                               positions) -> int:
        p = params.to_c()
        pos = np.ascontiguousarray(np.asarray(positions, dtype=np.uint64))
        rid = _U64()
        check(self.ctx.handle, self.L.bz_server_submit_commit_open(
            self.h, host_ptr, n_words, ctypes.byref(p), ptr(pos) if len(pos) else None, len(pos),
            ctypes.byref(rid)))
        return rid.value

    def next_done(self, cap: int = 64, timeout_us: int = 0) -> list[tuple[int, int]]:
        """(id, state entered) for the state changes since the previous call
        (bounded wait)."""
        ids = np.zeros(max(cap, 1), np.uint64)
        states = np.zeros(max(cap, 1), np.int32)
        n = _S()
        check(self.ctx.handle, self.L.bz_server_next_done(self.h, ptr(ids), ptr(states), cap,
                                                          ctypes.byref(n), int(timeout_us)))
        return [(int(i), int(st)) for i, st in zip(ids[:n.value], states[:n.value])]

    def submit_open(self, rid: int, positions) -> None:
        pos = np.ascontiguousarray(np.asarray(positions, dtype=np.uint64))
        check(self.ctx.handle, self.L.bz_server_submit_open(self.h, rid, ptr(pos) if len(pos) else None,
                                                            len(pos)))

    def state(self, rid: int) -> int:
        s = ctypes.c_int()
        check(self.ctx.handle, self.L.bz_server_poll(self.h, rid, ctypes.byref(s)))
        return s.value

    def wait(self, rid: int, state: int, timeout_ms: int = 60000) -> None:
        check(self.ctx.handle, self.L.bz_server_wait(self.h, rid, state, timeout_ms))
        if state >= COMMITTED:
            self._keep.pop(rid, None)

    def root(self, rid: int) -> bytes:
        out = (ctypes.c_uint8 * 32)()
        check(self.ctx.handle, self.L.bz_server_root(self.h, rid, out))
        return bytes(out)

    def open_result(self, rid: int, lanes: int):
        nr, nh = _S(), _S()
        check(self.ctx.handle, self.L.bz_server_open_result(self.h, rid, None, 0, None, 0,
                                                            ctypes.byref(nr), ctypes.byref(nh)))
        rows = np.zeros((max(nr.value, 1), lanes, 2), np.uint64)
        proof = np.zeros((max(nh.value, 1), 32), np.uint8)
        check(self.ctx.handle, self.L.bz_server_open_result(self.h, rid, ptr(rows), rows.size,
                                                            ptr(proof), proof.shape[0],
                                                            ctypes.byref(nr), ctypes.byref(nh)))
        return rows[:nr.value], proof[:nh.value]

    def times(self, rid: int):
        t = np.zeros(5, np.int64)
        check(self.ctx.handle, self.L.bz_server_times(self.h, rid, ptr(t)))
        return t

    def release(self, rid: int):
        check(self.ctx.handle, self.L.bz_server_release(self.h, rid))
        self._keep.pop(rid, None)

    def stats(self):
        v = [_U64() for _ in range(5)]
        check(self.ctx.handle, self.L.bz_server_stats(self.h, *[ctypes.byref(x) for x in v]))
        keys = ("committed", "opened", "failed", "in_use", "queued")
        return {k: x.value for k, x in zip(keys, v)}
