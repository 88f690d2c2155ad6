"""Batched grand-product GKR prover on the GPU (C ABI bz_gkr_*), the Python
mirror of BitZ's ``gpgkr_prove`` over ``GrandProductCircuit::batched_eval``
(src/bitz/gkr.rs:80-125) and of ``Forest::prove`` (src/bitz/forest.rs:246).

The transcript is the caller's: an object with ``send(stage, [a, b])``
(absorb a prover message of two field elements) and ``challenge(stage)``
(the next challenge), stage ``ROUND`` (the reference's Stage::GkrRound) or
``CLOSE`` (Stage::GkrClose).  Field elements are (2,) uint64 arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .pcs import Context, DeviceArray, default_context

ROUND, CLOSE = 0, 1

_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                       ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64))


_P, _S, _I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int


def _lib():
    L = lib()
    L.bz_gkr_prove.argtypes = [_P, _P, _S, _S, _P, _CB, _P, _P, _P, _P]
    L.bz_gkr_prove_device.argtypes = [_P, _P, _S, _S, _P, _CB, _P, _P, _P, _P]
    L.bz_gkr_forest_prove.argtypes = [_P, _P, _P, _I, _I, _P, _CB, _P, _P, _P, _P]
    return L


def _callback(transcript, errors: list):
    def cb(_user, stage, msg, out):
        try:
            m = np.ctypeslib.as_array(msg, shape=(4,)).copy()
            transcript.send(stage, [m[0:2], m[2:4]])
            ch = np.asarray(transcript.challenge(stage), np.uint64).reshape(2)
            out[0], out[1] = int(ch[0]), int(ch[1])
            return 0
        except Exception as e:  # reported after the call returns
            errors.append(e)
            return 1
    return _CB(cb)


def _finish(ctx, rc, errors, log_n, groups, roots, point, claim):
    if errors:
        raise errors[0]
    check(ctx.handle, rc)
    return (roots, [point[i].copy() for i in range(log_n)], claim)


def prove(leaves, groups: int, point, transcript, ctx: Context | None = None):
    """(roots, little-endian leaf point, leaf claim) for ``leaves`` (host
    (n, 2) uint64, n a power of two, or a DeviceArray, which is overwritten)
    proved down from the claim point ``point`` (log2(groups) elements) on the
    ``groups`` roots."""
    ctx = ctx or default_context()
    L = _lib()
    n = leaves.n if isinstance(leaves, DeviceArray) else np.asarray(leaves).reshape(-1, 2).shape[0]
    log_n = n.bit_length() - 1
    pt = np.ascontiguousarray(np.asarray(point, np.uint64).reshape(-1, 2))
    pt_arg = ptr(pt) if pt.size else None
    roots = np.zeros((groups, 2), np.uint64)
    out_point = np.zeros((log_n, 2), np.uint64)
    claim = np.zeros(2, np.uint64)
    errors: list = []
    cb = _callback(transcript, errors)
    if isinstance(leaves, DeviceArray):
        rc = L.bz_gkr_prove_device(ctx.handle, leaves.ptr, n, groups, pt_arg, cb, None,
                                   ptr(roots), ptr(out_point), ptr(claim))
    else:
        a = np.ascontiguousarray(leaves, np.uint64).reshape(-1, 2)
        rc = L.bz_gkr_prove(ctx.handle, ptr(a), n, groups, pt_arg, cb, None, ptr(roots),
                            ptr(out_point), ptr(claim))
    return _finish(ctx, rc, errors, log_n, groups, roots, out_point, claim)


def forest_prove(packed, images, t: int, s: int, zeta, transcript,
                 ctx: Context | None = None):
    """Forest::prove from its inputs: ``packed`` (ceil(2^s / 64), 2^t)
    uint64 column-group words per row, ``images`` (2^t, 2), ``zeta`` s
    elements.  Returns (roots, little-endian leaf point, leaf claim)."""
    ctx = ctx or default_context()
    L = _lib()
    pk = np.ascontiguousarray(np.asarray(packed, np.uint64).reshape(-1, 1 << t))
    im = np.ascontiguousarray(np.asarray(images, np.uint64).reshape(1 << t, 2))
    z = np.ascontiguousarray(np.asarray(zeta, np.uint64).reshape(-1, 2))
    roots = np.zeros((1 << s, 2), np.uint64)
    out_point = np.zeros((t + s, 2), np.uint64)
    claim = np.zeros(2, np.uint64)
    errors: list = []
    cb = _callback(transcript, errors)
    rc = L.bz_gkr_forest_prove(ctx.handle, ptr(pk), ptr(im), t, s, ptr(z) if z.size else None,
                               cb, None, ptr(roots), ptr(out_point), ptr(claim))
    return _finish(ctx, rc, errors, t + s, 1 << s, roots, out_point, claim)


__all__ = ["ROUND", "CLOSE", "prove", "forest_prove"]
