"""GB300-native Ligerito / Reed-Solomon commitment path of BitZ.

The compute path is libbitzgpu.so (hand-written sm_103a CUDA behind the C ABI
in include/bitz_gpu.h); this package is the host-side mirror of the
reference's commit/open interface over that ABI.
"""
from ._lib import BzError, declared_symbols, lib, lib_path  # noqa: F401
from .pcs import (  # noqa: F401
    LOG_PACKING,
    Commitment,
    Context,
    DeviceArray,
    HashKind,
    LigeroWitness,
    PcsParams,
    ProverData,
    BatchPlan,
    chacha_words,
    commit,
    commit_batch,
    default_context,
    ligero_commit,
)
from .transcript import Blake3Transcript, ZincChallenger, blake3_xof, pow_first_nonce  # noqa: F401,E402
from .opening import L0Config, L0Opening, LigeritoConfig, open_l0, prove  # noqa: F401,E402
from . import codec  # noqa: F401,E402
from .binary_pcs import BinaryPcs, BitMleOpening, Round0Prover  # noqa: F401,E402
from . import ingest  # noqa: F401,E402
from . import shard  # noqa: F401,E402
from . import gkr  # noqa: F401,E402
