"""Lane-sharded BLAKE3 commit: one commit split over the lanes of its matrix,
one rank per GPU.

The reference commits on one machine; this is the multi-GPU form of its
``pcs::commit::commit`` (flock-core/src/pcs/commit.rs:180-315).  Every lane's
NTT is independent (flock-core/src/ntt/additive_ntt_f128.rs:176-191) and a
BLAKE3 leaf is the tree over its 1 KiB chunks of 64 lanes, each chunk's index
in the leaf being its counter (flock-core/src/merkle.rs:160-201).  So rank r of
``world`` (a power of two, at least 64 lanes per rank) encodes its lanes,
reduces each of its rows to the CV of the run of chunks it holds, and the
ranks exchange those CVs (32 bytes per position per rank: the only
collective).  Every rank then merges them into the leaf CVs and builds the
Merkle tree, whose root is the whole commit's root.  Opened rows are gathered
the same way, one lane slice per rank.  SHA-256 commits are not sharded (their
leaves hash each row sequentially over every lane): use replicas.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .pcs import (Commitment, Context, DeviceArray, HashKind, PcsParams, ProverData,
                  default_context)


def _log2_world(world: int) -> int:
    if world < 1 or world & (world - 1):
        raise ValueError("world must be a power of two")
    return world.bit_length() - 1


def shard_params(params: PcsParams, world: int) -> PcsParams:
    """The shape one rank commits: 1/world of the lanes, same code length."""
    lw = _log2_world(world)
    if params.merkle_hash != HashKind.BLAKE3:
        raise ValueError("only BLAKE3 commits shard by lanes")
    if params.log_batch_size - lw < 6:
        raise ValueError("each rank needs at least 64 lanes")
    return PcsParams(params.m - lw, params.log_inv_rate, params.log_batch_size - lw,
                     params.merkle_hash)


def lane_shard(msg: np.ndarray, params: PcsParams, world: int, rank: int) -> np.ndarray:
    """Rank's message shard, compact: shard[col * Ls + j] = msg[col * L + rank * Ls + j]."""
    L = params.num_ntts()
    ls = L // world
    m = np.asarray(msg, np.uint64).reshape(-1, L, 2)
    return np.ascontiguousarray(m[:, rank * ls:(rank + 1) * ls]).reshape(-1, 2)


def commit_shard(msg_shard, params: PcsParams, world: int, rank: int,
                 ctx: Context | None = None) -> ProverData:
    """Rank's share of the commit (bz_commit_shard): its codeword lanes, and as
    leaves the CV of each position's run of chunks.  ``params`` are the whole
    commit's."""
    ctx = ctx or default_context()
    sp = shard_params(params, world)
    p = params.to_c()
    h = ctypes.c_void_p()
    L = lib()
    if isinstance(msg_shard, DeviceArray):
        check(ctx.handle, L.bz_commit_shard_device(ctx.handle, msg_shard.ptr, msg_shard.n,
                                                   ctypes.byref(p), world, rank, ctypes.byref(h)))
        check(ctx.handle, L.bz_ctx_synchronize(ctx.handle))
    else:
        a = np.ascontiguousarray(msg_shard, dtype=np.uint64).reshape(-1, 2)
        check(ctx.handle, L.bz_commit_shard(ctx.handle, ptr(a), a.shape[0], ctypes.byref(p),
                                            world, rank, ctypes.byref(h)))
    return ProverData(h, sp, ctx)


def leaf_cvs(pd: ProverData) -> np.ndarray:
    """The (n_leaves, 32) leaves of a commitment's tree."""
    n = pd.params.n_leaves()
    out = np.zeros((n, 32), np.uint8)
    check(pd.ctx.handle, lib().bz_commitment_leaf_cvs(pd._h(), ptr(out), n))
    return out


def merkle_from_shards(cvs: np.ndarray, params: PcsParams, ctx: Context | None = None):
    """(Commitment, tree-only ProverData) from every rank's leaf CVs
    ((world, n_leaves, 32), rank order)."""
    ctx = ctx or default_context()
    cvs = np.ascontiguousarray(cvs, np.uint8)
    world = cvs.shape[0]
    p = params.to_c()
    h = ctypes.c_void_p()
    root = (ctypes.c_uint8 * 32)()
    check(ctx.handle, lib().bz_merkle_from_shards(ctx.handle, ptr(cvs), world, ctypes.byref(p),
                                                  ctypes.byref(h), root))
    return Commitment(bytes(root), params), ProverData(h, params, ctx)


# ---- the exchange (torch.distributed: NCCL between GPUs, gloo on CPU) ------
def _all_gather(arr: np.ndarray, group=None) -> np.ndarray:
    """(world,) + arr.shape, in rank order.  Sent as raw bytes (gloo has no
    unsigned 64-bit tensors)."""
    import torch
    import torch.distributed as dist

    arr = np.ascontiguousarray(arr)
    world = dist.get_world_size(group)
    dev = torch.device("cpu")
    if dist.get_backend(group) == "nccl":
        dev = torch.device("cuda", torch.cuda.current_device())
    t = torch.from_numpy(arr.reshape(-1).view(np.uint8).copy()).to(dev)
    outs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(outs, t, group=group)
    return np.stack([o.cpu().numpy().view(arr.dtype).reshape(arr.shape) for o in outs])


def sharded_root(shard_cvs: np.ndarray, group=None, combine=None):
    """Exchange this rank's (n_leaves, 32) CVs and build the tree from all of
    them with ``combine`` (default: merkle_from_shards on this rank's GPU)."""
    allc = _all_gather(shard_cvs, group)
    return combine(allc)


def gather_rows(rows_slice: np.ndarray, group=None) -> np.ndarray:
    """Whole opened rows (q, L, 2) from every rank's (q, L/world, 2) slice."""
    allr = _all_gather(rows_slice, group)          # (world, q, Ls, 2)
    w, q, ls, _ = allr.shape
    return np.ascontiguousarray(allr.transpose(1, 0, 2, 3)).reshape(q, w * ls, 2)


class ShardedCommit:
    """This rank's part of a lane-sharded commit: its codeword lanes (rows),
    and the whole tree (root, multi-proofs)."""

    def __init__(self, commitment: Commitment, shard: ProverData, tree: ProverData, group):
        self.commitment = commitment
        self.shard = shard
        self.tree = tree
        self.group = group

    @property
    def root(self) -> bytes:
        return self.commitment.root

    def rows(self, positions) -> np.ndarray:
        """Whole opened rows: every rank calls this with the same positions."""
        return gather_rows(self.shard.rows(positions), self.group)

    def multi_proof(self, positions) -> np.ndarray:
        return self.tree.multi_proof(positions)

    def free(self):
        self.shard.free()
        self.tree.free()


def commit_lane_sharded(msg_shard, params: PcsParams, group=None,
                        ctx: Context | None = None) -> ShardedCommit:
    """One commit over every rank of ``group`` (one GPU each): this rank commits
    its lane shard, the ranks exchange per-position CVs, and every rank builds
    the whole tree."""
    import torch.distributed as dist

    ctx = ctx or default_context()
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    shard = commit_shard(msg_shard, params, world, rank, ctx)
    c, tree = sharded_root(leaf_cvs(shard), group,
                           combine=lambda allc: merkle_from_shards(allc, params, ctx))
    return ShardedCommit(c, shard, tree, group)


__all__ = ["shard_params", "lane_shard", "commit_shard", "leaf_cvs", "merkle_from_shards",
           "sharded_root", "gather_rows", "ShardedCommit", "commit_lane_sharded"]
