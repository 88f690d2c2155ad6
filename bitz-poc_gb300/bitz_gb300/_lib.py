"""ctypes binding of libbitzgpu.so (the C ABI in include/bitz_gpu.h).

The library is the product: every call below goes to CUDA kernels.  There is
no CPU fallback -- if the shared library is missing or no GPU is visible the
calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_P = ctypes.c_void_p
_S = ctypes.c_size_t
_I = ctypes.c_int
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_PP = ctypes.POINTER(ctypes.c_void_p)


class BzError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"bitz_gpu status {status}: {msg}")
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [("log_msg_len", _U32), ("log_inv_rate", _U32), ("log_batch_size", _U32),
                ("hash_kind", _U32)]


_lib = None

_SIGS = {
    "bz_status_string": (ctypes.c_char_p, [_I]),
    "bz_last_error": (ctypes.c_char_p, [_P]),
    "bz_abi_version": (_I, []),
    "bz_ctx_create": (_I, [_I, _U64, _PP]),
    "bz_ctx_destroy": (_I, [_P]),
    "bz_ctx_stream": (_P, [_P]),
    "bz_ctx_synchronize": (_I, [_P]),
    "bz_ctx_memory": (_I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "bz_device_alloc": (_I, [_P, _S, _PP]),
    "bz_device_free": (_I, [_P, _P]),
    "bz_memcpy_h2d": (_I, [_P, _P, _P, _S]),
    "bz_memcpy_d2h": (_I, [_P, _P, _P, _S]),
    "bz_host_alloc_pinned": (_I, [_S, _PP]),
    "bz_host_free_pinned": (_I, [_P]),
    "bz_timer_begin": (_I, [_P]),
    "bz_timer_end": (_I, [_P, ctypes.POINTER(ctypes.c_float)]),
    "bz_kernel_launches": (_U64, [_P]),
    "bz_commit": (_I, [_P, _P, _S, ctypes.POINTER(Params), _PP, _P]),
    "bz_commit_device": (_I, [_P, _P, _S, ctypes.POINTER(Params), _PP, _P]),
    "bz_commit_device_async": (_I, [_P, _P, _S, ctypes.POINTER(Params), _PP]),
    "bz_commit_async": (_I, [_P, _P, _S, ctypes.POINTER(Params), _PP]),
    "bz_commitment_root": (_I, [_P, _P]),
    "bz_commitment_params": (_I, [_P, ctypes.POINTER(Params)]),
    "bz_commitment_device_ptrs": (_I, [_P, _PP, _PP]),
    "bz_commitment_copy_codeword": (_I, [_P, _P, _S]),
    "bz_commitment_copy_tree": (_I, [_P, _P, _S]),
    "bz_commitment_rows": (_I, [_P, _P, _S, _P]),
    "bz_commitment_multiproof": (_I, [_P, _P, _S, _P, _S, ctypes.POINTER(_S)]),
    "bz_commitment_free": (_I, [_P]),
    "bz_commit_profile": (_I, [_P, _P, _S, ctypes.POINTER(Params), _S, _P, _P,
                               ctypes.POINTER(_S), _P]),
    "bz_ligero_commit_device": (_I, [_P, _P, _U32, _U32, _U32, _U32, _PP, _P]),
    "bz_commit_batch_device": (_I, [_P, _S, _P, ctypes.POINTER(Params), _PP, _P, _I]),
    "bz_fold_and_msg_lsb": (_I, [_P, _P, _P, _S, _P, _P, _P, _P, _P]),
    "bz_fold_and_msg_lsb_static": (_I, [_P, _P, _S, _P, _P, _P, _P, _P]),
    "bz_round_msg_lsb": (_I, [_P, _P, _P, _S, _P, _P]),
    "bz_fold_gate_check": (_I, [_P, _P, _P, _S, _P, _P, _P, _I, _U64, _P, _P]),
    "bz_partial_eval_lsb": (_I, [_P, _P, _S, _P, _S, _P]),
    "bz_build_eq_lsb": (_I, [_P, _P, _S, _P]),
    "bz_sv_fold": (_I, [_P, _P, _P, _S, _P]),
    "bz_phi_from_words": (_I, [_P, _P, _S, _P, _P]),
    "bz_chacha_fill_device": (_I, [_P, _U64, _U64, _P, _S]),
    "bz_chacha_fill_host": (_I, [_U64, _U64, _P, _S, _I]),
    "bz_transcript_create": (_I, [_PP]),
    "bz_transcript_clone": (_I, [_P, _PP]),
    "bz_transcript_destroy": (_I, [_P]),
    "bz_transcript_absorb": (_I, [_P, _P, _S]),
    "bz_transcript_absorb_slice": (_I, [_P, _P, _S]),
    "bz_transcript_challenge": (_I, [_P, _P, _S]),
    "bz_transcript_sample_f128": (_I, [_P, _P]),
    "bz_transcript_observe_f128": (_I, [_P, _P]),
    "bz_transcript_fill_sampling_bytes": (_I, [_P, _P, _S]),
    "bz_transcript_state_digest": (_I, [_P, _P]),
    "bz_blake3_xof": (_I, [_P, _S, _P, _S]),
    "bz_pow_first_nonce": (_I, [_P, _P, _S, _U32, _U64, _U64, ctypes.POINTER(_U64)]),
    "bz_transcript_grind_pow": (_I, [_P, _P, _U32, ctypes.POINTER(_U64)]),
    "bz_transcript_verify_pow": (_I, [_P, _U64, _U32, ctypes.POINTER(_I)]),
    "bz_ligerito_open_l0": (_I, [_P, _P, _P, _P, _P, _P, _P, _PP]),
    "bz_l0_opening_sizes": (_I, [_P, _P]),
    "bz_l0_opening_copy": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "bz_l0_opening_take_rows": (_I, [_P, _PP, ctypes.POINTER(ctypes.POINTER(ctypes.c_uint64))]),
    "bz_rows_free": (_I, [_P]),
    "bz_l0_opening_level1": (_P, [_P]),
    "bz_l0_opening_folded": (_I, [_P, _PP, _PP, ctypes.POINTER(_S)]),
    "bz_l0_opening_free": (_I, [_P]),
    "bz_l0_opening_ood_values": (_I, [_P, _P]),
    "bz_ligerito_prove": (_I, [_P, _P, _P, _P, _P, _P, _P, _PP]),
    "bz_pcs_prove_round0": (_I, [_P, _P, _P, _S, _U32, _PP]),
    "bz_round0_get": (_I, [_P, _P, ctypes.POINTER(_I), ctypes.POINTER(_U64),
                           ctypes.POINTER(_U32)]),
    "bz_round0_point": (_I, [_P, _P]),
    "bz_round0_free": (_I, [_P]),
    "bz_pcs_ring_switch": (_I, [_P, _P, _P, _S, _P, _P, _P, _P]),
    "bz_pcs_open_basis": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _PP]),
    "bz_pcs_open_bit_mle": (_I, [_P, _P, _P, _P, _P, _P, _S, _P, _P, _PP]),
    "bz_ligerito_proof_encode": (_I, [_P, _P, _S, ctypes.POINTER(_S)]),
    "bz_ligerito_proof_decode": (_I, [_P, _S, _PP]),
    "bz_ligerito_proof_view_of": (_I, [_P, _P]),
    "bz_ligerito_proof_free": (_I, [_P]),
    "bz_writer_create": (_I, [_PP]),
    "bz_writer_destroy": (_I, [_P]),
    "bz_writer_len": (_I, [_P, _U64]),
    "bz_writer_gf": (_I, [_P, _P]),
    "bz_writer_bytes": (_I, [_P, _P, _S]),
    "bz_writer_data": (_I, [_P, _P, ctypes.POINTER(_S)]),
    "bz_write_round0": (_I, [_P, _P, _I, _U64]),
    "bz_write_ring_switch": (_I, [_P, _P]),
    "bz_write_ligerito": (_I, [_P, _P]),
    "bz_reader_create": (_I, [_P, _S, _PP]),
    "bz_reader_destroy": (_I, [_P]),
    "bz_reader_remaining": (_S, [_P]),
    "bz_reader_len": (_I, [_P, ctypes.POINTER(_U64)]),
    "bz_reader_gf": (_I, [_P, _P]),
    "bz_reader_take": (_I, [_P, _S, _P]),
    "bz_read_round0": (_I, [_P, _P, ctypes.POINTER(_I), ctypes.POINTER(_U64)]),
    "bz_read_ring_switch": (_I, [_P, _P]),
    "bz_read_ligerito": (_I, [_P, _PP]),
    "bz_repack_leaf_bits": (_I, [_P, _P, _U32, _U32, _P]),
    "bz_pack_columns_from_rows": (_I, [_P, _P, _U32, _U32, _P]),
    "bz_rows_from_packed_cols": (_I, [_P, _P, _U32, _U32, _P]),
    "bz_commit_rows": (_I, [_P, _P, _U32, _U32, _U32, _U32, _U32, _PP, _P]),
    "bz_commit_shard": (_I, [_P, _P, _S, ctypes.POINTER(Params), _U32, _U32, _PP]),
    "bz_gkr_prove": (_I, [_P, _P, _S, _S, _P, _P, _P, _P, _P, _P]),
    "bz_gkr_prove_device": (_I, [_P, _P, _S, _S, _P, _P, _P, _P, _P, _P]),
    "bz_gkr_forest_prove": (_I, [_P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _P]),
    "bz_commit_shard_device": (_I, [_P, _P, _S, ctypes.POINTER(Params), _U32, _U32, _PP]),
    "bz_commitment_leaf_cvs": (_I, [_P, _P, _S]),
    "bz_merkle_from_shards": (_I, [_P, _P, _U32, ctypes.POINTER(Params), _PP, _P]),
    "bz_autotune": (_I, [_P, ctypes.POINTER(Params), _I, ctypes.POINTER(_U32)]),
    "bz_schedule_get": (_I, [_P, ctypes.POINTER(Params), ctypes.POINTER(_U32)]),
    "bz_schedule_set": (_I, [_P, ctypes.POINTER(Params), _U32]),
}


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise OSError(f"{path} not built")
            _build.build()
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def declared_symbols() -> list[str]:
    """Every function the public header declares."""
    import re

    hdr = os.path.join(os.path.dirname(_build.ROOT), "include")
    names = []
    for fn in sorted(os.listdir(hdr)):
        if fn.endswith(".h"):
            with open(os.path.join(hdr, fn)) as fh:
                text = fh.read()
            names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(bz_[a-z0-9_]+)\s*\(", text,
                                re.M)
    return sorted(set(names))


def check(ctx, status: int):
    if status != 0:
        L = lib()
        msg = L.bz_status_string(status).decode()
        if ctx is not None:
            detail = L.bz_last_error(ctx)
            if detail:
                msg += ": " + detail.decode()
        raise BzError(status, msg)


def ptr(a: np.ndarray):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(ctypes.c_void_p)
