"""Benchmark: committed field elements per second for the Ligerito / RS commit
(additive NTT + Merkle, bit-exact) of a 2^24-element polynomial laid out as a
2^12 x 2^12 matrix, rate 1/4, BLAKE3 Merkle tree over 16384 columns.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on stdout (rank 0).  Under torchrun each rank commits its own
polynomial (independent objects, no data-path collective: weak scaling); the
timed region is bracketed by a barrier and a device synchronize, and the
maximum over ranks is reported.  The reference arm times the CPU
restatement of the reference's commit (oracle/, "port": the reference is Rust
and no Rust toolchain exists on the machine) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

# One hardware work queue per stream (CUDA's default is 8 per device, read once
# before the process's first CUDA call): the server's slot streams, the batch
# plan's branches and the context's own streams would otherwise share queues,
# and a small request's kernels could wait behind a large one's in the same
# queue whatever their stream priorities.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "bitz-poc_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

LOG_N = 24          # 2^24 committed GF(2^128) elements
LOG_LANES = 12      # 2^12 matrix rows (interleaved lanes) x 2^12 columns
LOG_INV_RATE = 2    # rate 1/4 -> 16384 codeword columns (Merkle leaves)
HASH = 1            # BLAKE3
SEED = 1
METRIC = "committed field elems/sec (NTT+Merkle, bit-exact) at 2^24"
UNIT = "elems/s"
WORKLOAD = {
    "workload": "ligerito_rs_commit_2^24",
    "matrix": "2^12 x 2^12 GF(2^128)",
    "rate": "1/4",
    "merkle_leaves": 16384,
    "hash": "blake3",
    "inputs": "ChaCha20 seed 1 (+rank), uniform GF(2^128)",
    "l2": "inputs larger than L2: 256 MiB message, 1 GiB codeword per step",
}
MSG_BYTES = 16 << LOG_N
CPU_PORT_SAMPLE = ("{what} by oracle/oracle.c on all host threads: a C restatement of the "
                   "reference's commit with its parallel structure (top NTT layers fused in "
                   "pairs, deep layers per cache-resident 2 MiB sub-group, persistent thread "
                   "pool, PMULL multiplies on aarch64), not the reference's own Rust code "
                   "(no Rust toolchain on either machine); its BLAKE3 is a portable scalar "
                   "restatement, where the reference's crate hashes with NEON/AVX")
ALG_BYTES_PER_WORD = 16 + (16 << LOG_INV_RATE)   # read message + write codeword
SCHED_PIPE_BITS = 3 << 10                         # pipeline chunk count of a schedule
# One GF(2^128) multiply by a block twiddle = 16 byte-table lookups of 16 B.
T16_BYTES_PER_MUL = 16 * 16
SMEM_BYTES_PER_CLK_PER_SM = 128
# DRAM bytes (read + write) per codeword byte of one launch, from ncu
# captures of the same kernels on GB300 (dram__bytes_read.sum +
# dram__bytes_write.sum), with the profile they come from.
NCU_TRAFFIC_PER_CW_BYTE = {
    "ntt_pass8_first": (1.424, "profiles/launches_commit_2e24.md"),
    "ntt_pass8": (1.941, "profiles/launches_commit_2e24.md (both in-place byte-table passes)"),
    "ntt_pass8_nw": (1.940, "profiles/launches_commit_2e24.md"),
    "b3_leaves_chunked": (1.057, "profiles/launches_commit_2e24.md"),
    # radix-4 schedules sweep the codeword the same way: one read and one
    # write in place, the first pass reading the message instead
    "ntt_table_pass2_first": (1.424, "profiles/launches_commit_2e24.md (a first sweep)"),
    "ntt_table_pass2": (1.941, "profiles/launches_commit_2e24.md (an in-place sweep)"),
    "ntt_table_pass2_nw": (1.940, "profiles/launches_commit_2e24.md (an in-place sweep)"),
}


def table_pass_lookup_bytes(kernel: str, layer: int, log_positions_lanes: int) -> int | None:
    """Shared-memory bytes read by the twiddle multiplies of one table pass
    over 2^log_positions_lanes codeword elements starting at `layer` (16
    lookups of 16 B per product with either table layout: sixteen tables of
    one byte position each, or eight tables serving both 64-bit halves).

    A radix-4 pass multiplies each quad 4 times (t_o twice, then t_a and
    t_b), a radix-2 pass each pair once.  Block 0 of every layer has a zero
    twiddle (the span of no evaluation is 0), so its quads skip the t_o and
    t_a products and its pairs skip theirs."""
    n = 1 << log_positions_lanes
    if kernel.endswith("_nw"):
        return None   # compact 4-byte tables for narrow twiddles: not this model
    if kernel.startswith("ntt_pass8"):
        # radix-8: 12 products per octet; block 0's seven zero twiddles skip
        # 4 + 2 + 1 of them in the first super-block
        octets = n // 8
        muls = 12 * octets - 7 * (octets >> layer)
        return muls * T16_BYTES_PER_MUL
    if kernel.startswith("ntt_table_pass2"):
        quads = n // 4
        muls = 4 * quads - 3 * (quads >> layer)
    else:
        pairs = n // 2
        muls = pairs - (pairs >> layer)
    return muls * T16_BYTES_PER_MUL


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class _Dist:
    def __init__(self, ws, local):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch
            import torch.distributed as dist

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend)
            self.dist = dist
            self.torch = torch
            self.dev = torch.device("cuda", local) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class _Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout_s: float = 5.0):
        """Block until the sampler produced a line, so samples cover what follows."""
        t0 = time.perf_counter()
        while self.proc and not self.lines and time.perf_counter() - t0 < timeout_s:
            time.sleep(0.01)
        self.lines.clear()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(n_threads: int, log_n: int = LOG_N):
    """The oracle commit (CPU restatement of the reference) on a full 2^24
    commit with all host threads; elements per second.  With several threads
    the oracle runs the reference's parallel structure (top NTT layers fused
    in pairs, deep layers per cache-resident 2 MiB sub-group, a persistent
    thread pool; PMULL multiplies on aarch64), not its per-layer form.  Also
    times the oracle's recursive Ligerito proof of that commitment with the
    opening leg's configuration (its folds run on one thread)."""
    from oracle import oracle as O
    from oracle.ligerito import LigeritoConfig, prove
    from oracle.transcript import Blake3Transcript, ZincChallenger

    O.build()
    msg = O.chacha_words(SEED, 1 << log_n)
    t0 = time.perf_counter()
    cw, tree, root = O.commit(msg, LOG_INV_RATE, LOG_LANES, HASH, n_threads=n_threads)
    dt = time.perf_counter() - t0
    basis = O.chacha_words(77, 1 << log_n)
    t = Blake3Transcript()
    t.absorb_slice(b"bench opening")
    t1 = time.perf_counter()
    prove(ZincChallenger(t), LigeritoConfig(**open_config(LOG_LANES)), msg, basis, [1, 2], cw,
          tree, root)
    open_ms = (time.perf_counter() - t1) * 1e3
    # the 2^20-word bit-MLE opening (round 0 + open_bit_mle), as the GPU leg
    from oracle.binary_pcs import open_bit_mle, prove_round0

    m = 20
    p20 = O.chacha_words(0, 1 << m)
    cw20, tree20, root20 = O.commit(p20, 2, 10, HASH, n_threads=n_threads)
    point = np.random.default_rng(0).integers(0, 2**64, (m + 7, 2), dtype=np.uint64)
    t2 = Blake3Transcript()
    t2.absorb_slice(root20)
    t3 = time.perf_counter()
    r0 = prove_round0(t2, p20, BIT_MLE_ROUND0_BITS)
    open_bit_mle(t2, LigeritoConfig(**BIT_MLE_CONFIG), p20, cw20, tree20, root20, r0, point)
    bit_mle_ms = (time.perf_counter() - t3) * 1e3
    return (1 << log_n) / dt, dt, root, open_ms, bit_mle_ms


def cpu_gkr_ms(t: int = 12, s: int = 10) -> float:
    """The oracle's dense GKR prover (a CPU restatement of BitZ's gpgkr_prove,
    its field arithmetic in C, its loops in numpy) on the same 2^(t+s)-leaf
    forest as the GPU leg's first size, in ms."""
    from oracle import gkr as G

    rng = np.random.default_rng(77 + t)
    rows, cols = 1 << t, 1 << s
    packed = rng.integers(0, 2**64, ((cols + 63) // 64, rows), dtype=np.uint64)
    images = rng.integers(0, 2**64, (rows, 2), dtype=np.uint64)
    zeta = [rng.integers(0, 2**64, 2, dtype=np.uint64) for _ in range(s)]
    t0 = time.perf_counter()
    leaves = G.forest_leaves(packed, images, t, s)
    _, wit = G.batched_eval(leaves, cols)
    tr = G.HashChallenges(b"gkr-bench")
    G.prove(tr.send, tr.challenge, zeta, wit)
    return (time.perf_counter() - t0) * 1e3


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    msg = O.chacha_words(SEED, 1 << LOG_N)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.commit(msg, LOG_INV_RATE, LOG_LANES, HASH, n_threads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = args.steps * (1 << LOG_N) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (GF(2^128))",
        "data": "synthetic", "config": dict(WORKLOAD, parallelism=f"replicas{ws}"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": CPU_PORT_SAMPLE.format(what="full 2^24-element commit per "
                                                                   "step")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, ws, rank, local):
    import numpy as np

    import bitz_gb300 as bz
    from bitz_gb300 import _lib

    D = _Dist(ws, local)
    ctx = bz.Context(local)
    L = _lib.lib()
    params = bz.PcsParams(LOG_N + 7, LOG_INV_RATE, LOG_LANES, HASH)
    pc = params.to_c()
    import ctypes

    msg = bz.DeviceArray.chacha(SEED + rank, 1 << LOG_N, ctx)
    if args.schedule is not None:
        ctx.set_schedule(params, int(args.schedule, 0))
        schedule = ctx.schedule(params)
    else:
        schedule = ctx.autotune(params, reps=2) if not args.no_autotune else ctx.schedule(params)

    def one_commit():
        h = ctypes.c_void_p()
        _lib.check(ctx.handle, L.bz_commit_device_async(ctx.handle, msg.ptr, 1 << LOG_N,
                                                        ctypes.byref(pc), ctypes.byref(h)))
        root = (ctypes.c_uint8 * 32)()
        _lib.check(ctx.handle, L.bz_commitment_root(h, root))
        L.bz_commitment_free(h)
        return bytes(root)

    # parity of the benchmarked output against the committed oracle root
    root0 = one_commit()
    with open(os.path.join(REPO, "tests", "golden", "roots.json")) as fh:
        golden = {(e["log_msg_len"], e["seed"], e["hash"]): e["root"]
                  for e in json.load(fh)["roots"]}
    exp = golden.get((LOG_N, SEED + rank, "blake3"))
    parity = None if exp is None else (root0.hex() == exp)
    if parity is False:
        raise SystemExit(f"benchmarked commit root {root0.hex()} != oracle root {exp}")

    for _ in range(max(args.warmup, 3) - 1):
        one_commit()

    # ---- device-resident timed region -----------------------------------
    launches0 = ctx.kernel_launches()
    clocks = _Clocks(local)
    clocks.start()
    clocks.wait_first()
    D.barrier()
    ctx.synchronize()
    step_ms = []
    ctx.timer_begin()
    t_all0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.timer_begin()
        one_commit()
        step_ms.append(ctx.timer_end())
    ctx.synchronize()
    wall = time.perf_counter() - t_all0
    D.barrier()
    clk = clocks.stop()
    launches = ctx.kernel_launches() - launches0
    total_ms = sum(step_ms)
    total_ms = D.max(total_ms)
    value = ws * args.steps * (1 << LOG_N) / (total_ms / 1e3)

    if args.only_commit or args.only_open:
        if rank == 0:
            line = {"metric": METRIC, "value": value, "unit": UNIT, "log_n": LOG_N,
                    "ms_per_step": total_ms / args.steps, "schedule": schedule,
                    "root": root0.hex()}
            if args.only_open:
                line["opening"] = _bench_open(ctx, bz, msg, params)
            print(json.dumps(line), flush=True)
        msg.free()
        ctx.close()
        D.close()
        return 0

    # ---- end to end through the C ABI with host buffers ----------------
    hp = ctypes.c_void_p()
    _lib.check(None, L.bz_host_alloc_pinned(MSG_BYTES, ctypes.byref(hp)))
    _lib.check(None, L.bz_chacha_fill_host(SEED + rank, 0, hp, 1 << LOG_N, os.cpu_count() or 1))

    def e2e_commit():
        h = ctypes.c_void_p()
        root = (ctypes.c_uint8 * 32)()
        _lib.check(ctx.handle, L.bz_commit(ctx.handle, hp, 1 << LOG_N, ctypes.byref(pc),
                                           ctypes.byref(h), root))
        L.bz_commitment_free(h)
        return bytes(root)

    def e2e_submit():
        h = ctypes.c_void_p()
        _lib.check(ctx.handle, L.bz_commit_async(ctx.handle, hp, 1 << LOG_N, ctypes.byref(pc),
                                                 ctypes.byref(h)))
        return h

    def e2e_finish(h):
        root = (ctypes.c_uint8 * 32)()
        _lib.check(ctx.handle, L.bz_commitment_root(h, root))
        L.bz_commitment_free(h)
        return bytes(root)

    assert e2e_commit() == root0
    assert e2e_finish(e2e_submit()) == root0
    # every step: H2D of its own 256 MiB message from pinned memory, the commit
    # kernels and the D2H of its root; step i+1's upload overlaps step i's kernels
    D.barrier()
    ctx.synchronize()
    t_e2e0 = time.perf_counter()
    prev = e2e_submit()
    for _ in range(args.steps - 1):
        nxt = e2e_submit()
        assert e2e_finish(prev) == root0
        prev = nxt
    assert e2e_finish(prev) == root0
    e2e_ms = D.max((time.perf_counter() - t_e2e0) * 1e3)
    # the synchronous C-ABI call (no overlap) for reference
    ctx.synchronize()
    ctx.timer_begin()
    for _ in range(args.steps):
        e2e_commit()
    e2e_sync_ms = D.max(ctx.timer_end())
    e2e_value = ws * args.steps * (1 << LOG_N) / (e2e_ms / 1e3)
    L.bz_host_free_pinned(hp)

    out = None
    if rank == 0:
        # ---- per-kernel phase times and the roofline of the dominant kernel
        # (a pipelined schedule overlaps its kernels on two streams, so its
        # phase split is taken with the same kernels launched in sequence)
        prof_schedule = schedule & ~SCHED_PIPE_BITS
        if prof_schedule != schedule:
            ctx.set_schedule(params, prof_schedule)
        phases, proot = ctx.commit_profile(msg, params)
        if prof_schedule != schedule:
            ctx.set_schedule(params, schedule)
        assert proot == root0
        agg, lookup_bytes = {}, {}
        for name, ms in phases:
            kern, _, layer = name.partition("@")
            a = agg.setdefault(kern, [0, 0.0])
            a[0] += 1
            a[1] += ms
            if layer:
                lookup_bytes.setdefault(kern, []).append(
                    table_pass_lookup_bytes(kern, int(layer), LOG_N + LOG_INV_RATE))
        total_phase = sum(v[1] for v in agg.values())
        dom = max(agg.items(), key=lambda kv: kv[1][1])
        dom_name, (dom_n, dom_ms) = dom
        cw_bytes = 16 << (LOG_N + LOG_INV_RATE)
        # per launch: an in-place table pass reads and writes the codeword once
        if dom_name.endswith("_first"):
            alg_bytes = MSG_BYTES + cw_bytes
        elif dom_name.startswith("ntt"):
            alg_bytes = 2 * cw_bytes
        else:
            alg_bytes = cw_bytes
        peak, peak_kind = _peaks()
        achieved = alg_bytes / (dom_ms / dom_n / 1e3) / 1e9
        traffic = None
        if dom_name in NCU_TRAFFIC_PER_CW_BYTE:
            traffic = NCU_TRAFFIC_PER_CW_BYTE[dom_name][0] * cw_bytes
        smem = None
        if dom_name in lookup_bytes and None not in lookup_bytes[dom_name]:
            import torch

            sms = torch.cuda.get_device_properties(local).multi_processor_count
            mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
            lb = sum(lookup_bytes[dom_name]) / len(lookup_bytes[dom_name])
            s_ach = lb / (dom_ms / dom_n / 1e3) / 1e9
            s_peak = SMEM_BYTES_PER_CLK_PER_SM * sms * mhz * 1e6 / 1e9 if mhz else None
            smem = {"bound": "shared-memory pipe", "lookup_bytes_per_launch": lb,
                    "achieved": s_ach, "peak": s_peak, "unit": "GB/s",
                    "frac": s_ach / s_peak if s_peak else None,
                    "peak_source": f"nominal {SMEM_BYTES_PER_CLK_PER_SM} B/clk/SM x {sms} SMs x "
                                   f"median sampled SM clock {mhz} MHz"}
        commit_ms = statistics.median(step_ms)
        commit_gbs = ALG_BYTES_PER_WORD * (1 << LOG_N) / (commit_ms / 1e3) / 1e9
        # whole-commit DRAM traffic: every launch's ncu bytes per codeword byte
        # (the small tree levels excepted), when all of them were captured
        commit_traffic, missing = 0.0, []
        for kern, (n_l, _) in agg.items():
            if kern in NCU_TRAFFIC_PER_CW_BYTE:
                commit_traffic += n_l * NCU_TRAFFIC_PER_CW_BYTE[kern][0] * cw_bytes
            elif not kern.startswith("merkle_levels"):
                missing.append(kern)
        commit_traffic = None if missing else commit_traffic
        # every table pass's lookups over the commit time: the shared-memory
        # pipe bound of the whole NTT
        all_lb = [b for v in lookup_bytes.values() for b in v]
        commit_smem = None
        if all_lb and None not in all_lb and smem and smem["peak"]:
            ach = sum(all_lb) / (commit_ms / 1e3) / 1e9
            commit_smem = {"lookup_bytes": sum(all_lb), "achieved": ach, "peak": smem["peak"],
                           "unit": "GB/s", "frac": ach / smem["peak"],
                           "note": "wide-twiddle passes only; compact-table passes not counted"}

        # ---- batched (64 polys, log2 sizes U[16, 24], seed 3) vs plain -----
        batch = None
        if not args.skip_batch:
            batch = _bench_batch(ctx, bz, L, _lib, args)
        serve = None
        if not args.skip_serve:
            plain = batch["plain"]["value"] if batch else None
            serve = _bench_serve(ctx, bz, args, plain)
        shapes = None
        if not args.skip_shapes:
            shapes = _bench_shapes(ctx, bz)
        opening = None
        if not args.skip_open:
            opening = _bench_open(ctx, bz, msg, params)
        gkr = None
        if not args.skip_gkr:
            gkr = _bench_gkr(ctx, bz)

        # ---- CPU baseline (oracle, all host threads, one full commit) -----
        cpu = None
        if not args.skip_cpu:
            threads = os.cpu_count() or 1
            v, dt, croot, cpu_open_ms, cpu_bit_mle_ms = cpu_baseline(threads)
            assert croot == root0 or rank != 0 or SEED + rank != SEED
            cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": CPU_PORT_SAMPLE.format(
                       what=f"one full 2^24-element commit ({dt:.2f} s)"),
                   "prove_ms": cpu_open_ms, "bit_mle_2^20_round0_and_open_ms": cpu_bit_mle_ms}
            if not args.skip_gkr:
                cpu["gkr_forest_2^22_ms"] = cpu_gkr_ms()
        sorted_ms = sorted(step_ms)
        p99 = sorted_ms[min(len(sorted_ms) - 1, int(round(0.99 * (len(sorted_ms) - 1))))]
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64 (GF(2^128) carry-less)", "data": "synthetic",
            "config": dict(WORKLOAD, parallelism=f"replicas{ws}"),
            "parity": {"root_matches_oracle": parity, "root": root0.hex()},
            "latency_ms": {"p50": statistics.median(step_ms), "p99": p99,
                           "min": sorted_ms[0], "max": sorted_ms[-1]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": MSG_BYTES,
                    "d2h_bytes_per_step": 32, "api": "bz_commit_async + bz_commitment_root",
                    "pipelined": "upload of step i+1 overlaps the kernels of step i",
                    "sync_call_value": ws * args.steps * (1 << LOG_N) / (e2e_sync_ms / 1e3)},
            "roofline": {"bound": "hbm", "scope": "whole commit: 80 B per element (read "
                                                    "the message, write the codeword) over "
                                                    "the median commit time",
                         "achieved": commit_gbs, "peak": peak, "unit": "GB/s",
                         "frac": commit_gbs / peak, "traffic": commit_traffic,
                         "traffic_source": ("ncu DRAM bytes of every launch, "
                                            "profiles/launches_commit_2e24.md"
                                            if commit_traffic is not None else None),
                         "peak_source": peak_kind, "smem_commit": commit_smem,
                         "kernel": {"name": dom_name, "launches": dom_n,
                                    "achieved": achieved, "peak": peak, "unit": "GB/s",
                                    "frac": achieved / peak, "traffic": traffic,
                                    "traffic_source": (NCU_TRAFFIC_PER_CW_BYTE[dom_name][1]
                                                       if traffic is not None else None),
                                    "alg_bytes_per_launch": alg_bytes,
                                    "launch_ms": dom_ms / dom_n, "smem": smem},
                         "phase_schedule": prof_schedule},
            "phases_ms": {k: round(v[1], 4) for k, v in agg.items()},
            "phase_share": {k: round(v[1] / total_phase, 4) for k, v in agg.items()},
            "clocks": clk, "gpu_launches": launches, "wall_s": wall,
            "schedule": schedule, "batched": batch, "serving": serve, "shapes": shapes,
            "opening": opening, "gkr_forest": gkr, "cpu_baseline": cpu,
        }
        print(json.dumps(out), flush=True)
    msg.free()
    ctx.close()
    D.close()
    return 0


def _bench_batch(ctx, bz, L, _lib, args):
    """64 polynomials, log2 sizes uniform on [16, 24] (seed 3), square-ish
    2^floor(n/2) x 2^ceil(n/2) matrices, rate 1/4, per-shape autotuned
    schedules: the persistent plan (every commit as work items of one
    persistent kernel, launched through a CUDA graph), the graph plan (every
    commit's kernels in one CUDA graph over 4 parallel branches) and the same
    plan issued as stream launches, against the same 64 committed one at a
    time by the plain GPU path."""
    import numpy as np

    rng = np.random.default_rng(3)
    sizes = [int(x) for x in rng.integers(16, 25, 64)]
    params = [bz.PcsParams(n + 7, LOG_INV_RATE, n // 2, HASH) for n in sizes]
    for p in {(p.m, p.log_batch_size): p for p in params}.values():
        ctx.autotune(p, reps=1)
    msgs = [bz.DeviceArray.chacha(3000 + i, 1 << n, ctx) for i, n in enumerate(sizes)]
    total = int(sum(1 << n for n in sizes))
    reps = 5
    res = {}
    for mode, graph, branches in (("persistent", True, 0), ("graph", True, 4),
                                  ("stream_plan", False, 4)):
        plan = bz.BatchPlan(msgs, params, use_graph=graph, n_branches=branches, ctx=ctx,
                            persistent=mode == "persistent")
        plan.launch()
        plan.roots()
        ctx.synchronize()
        ctx.timer_begin()
        for _ in range(reps):
            plan.launch()
        ms = ctx.timer_end() / reps
        roots = plan.roots()
        plan.close()
        res[mode] = {"value": total / (ms / 1e3), "ms": ms}
        if mode == "persistent":
            persistent_roots = roots
    # plain: one commit at a time through bz_commit_device (root read per commit)
    import ctypes

    def plain_once():
        out = []
        for m, p in zip(msgs, params):
            c, pd = bz.commit(m, p, ctx)
            out.append(c.root)
            pd.free()
        return out

    plain_roots = plain_once()
    assert plain_roots == roots, "batched roots differ from one-at-a-time roots"
    assert plain_roots == persistent_roots, "persistent roots differ from one-at-a-time roots"
    ctx.synchronize()
    ctx.timer_begin()
    for _ in range(reps):
        plain_once()
    ms = ctx.timer_end() / reps
    res["plain"] = {"value": total / (ms / 1e3), "ms": ms}
    for m in msgs:
        m.free()
    return {"polys": 64, "total_elems": total, "unit": UNIT, "log2_sizes": sizes,
            "speedup_graph_vs_plain": res["plain"]["ms"] / res["graph"]["ms"],
            "speedup_persistent_vs_plain": res["plain"]["ms"] / res["persistent"]["ms"], **res}


def _bench_shapes(ctx, bz):
    """The 2^20-element (2^10 x 2^10) and 2^28-element (2^14 x 2^14, 16 GiB
    codeword resident in HBM) commits at rate 1/4, BLAKE3; NTT and Merkle
    phases timed separately (device events around every kernel)."""
    out = {}
    peak, _ = _peaks()
    for log_n, reps in ((20, 10), (28, 3)):
        p = bz.PcsParams(log_n + 7, LOG_INV_RATE, log_n // 2, HASH)
        m = bz.DeviceArray.chacha(log_n, 1 << log_n, ctx)
        sched = ctx.autotune(p, reps=1)
        # phases of a pipelined schedule are split with its kernels in sequence
        if sched & SCHED_PIPE_BITS:
            ctx.set_schedule(p, sched & ~SCHED_PIPE_BITS)
        best = None
        for _ in range(reps):
            phases, root = ctx.commit_profile(m, p)
            tot = sum(t for _, t in phases)
            if best is None or tot < best[0]:
                best = (tot, phases)
        tot, phases = best
        ntt = sum(t for n, t in phases if n.startswith("ntt") or n == "replicate_fill")
        mk = tot - ntt
        cw_bytes = 16 << (log_n + LOG_INV_RATE)
        out[f"2^{log_n}"] = {
            "value": (1 << log_n) / (tot / 1e3), "unit": UNIT, "ms": tot, "ntt_ms": ntt,
            "merkle_ms": mk, "schedule": sched, "phase_schedule": sched & ~SCHED_PIPE_BITS,
            "root": root.hex(),
            "commit_alg_gbs": ALG_BYTES_PER_WORD * (1 << log_n) / (tot / 1e3) / 1e9,
            "merkle_read_gbs": cw_bytes / (mk / 1e3) / 1e9, "hbm_peak_gbs": peak}
        m.free()
    return out


def open_config(log_lanes: int) -> dict:
    """The opening leg's ProverConfig for a 2^log_lanes x 2^log_lanes witness."""
    block1 = 1 << (log_lanes - log_lanes // 2 + 2)   # level-1 codeword length
    return dict(initial_k=log_lanes, recursive_ks=[log_lanes // 2],
                log_inv_rates=[LOG_INV_RATE, 2], queries=[148, min(148, block1 // 2)],
                grinding_bits=[16, 16], fold_grinding_bits=None, ood_samples=None,
                hash_kind=HASH)



OPEN_CONFIG_TEXT = ("recursive Ligerito, initial_k a, recursive_ks [a/2], log_inv_rates [2, 2], "
                    "queries [148, 148] (the rate-1/4 unique-decoding count), grinding_bits "
                    "[16, 16], no fold grinding, no OOD samples, BLAKE3")


def _bench_open(ctx, bz, msg, params):
    """Opening leg at 2^24 (2^12 lanes x 2^12 columns, rate 1/4): the whole
    recursive Ligerito proof of the resident commitment through
    bz_ligerito_prove (open_config), and its level-0 part alone through
    bz_ligerito_open_l0.  Host wall time of each call (they synchronize for
    every transcript squeeze), median of OPEN_REPS after one warm-up.  Also
    times the GPU proof-of-work search alone at 24 bits."""
    import numpy as np

    from bitz_gb300 import codec

    b = bz.DeviceArray.chacha(77, msg.n, ctx)
    c, pd = bz.commit(msg, params, ctx)
    cfg = bz.LigeritoConfig(**open_config(params.log_batch_size))

    def timed(fn, reps=OPEN_REPS + 1):
        # the previous rep's result is released outside the timed region
        ts, out, last = [], None, None
        for _ in range(reps):
            t = bz.Blake3Transcript()
            t.absorb_slice(b"bench opening")
            last = None
            ctx.synchronize()
            t0 = time.perf_counter()
            out = fn(t)
            ts.append(time.perf_counter() - t0)
            if hasattr(out, "free"):
                out.free()
            last, out = out, None
        return statistics.median(ts[1:]) * 1e3, min(ts[1:]) * 1e3, last

    prove_ms, prove_min, proof = timed(lambda t: bz.prove(t, pd, msg, b, [1, 2], cfg, ctx))
    prove_c_ms, _, _ = timed(lambda t: bz.prove(t, pd, msg, b, [1, 2], cfg, ctx, decode=False))
    blob = codec.encode_ligerito(proof)
    l0_cfg = bz.L0Config(initial_k=params.log_batch_size,
                         recursive_k0=params.log_batch_size // 2, log_inv_rate1=2,
                         grinding_bits0=16, queries0=148, hash_kind=HASH)
    l0_ms, l0_min, _ = timed(lambda t: bz.open_l0(t, pd, msg, b, [1, 2], l0_cfg, ctx))
    info = {"prove_ms": prove_ms, "prove_ms_min": prove_min, "prove_c_abi_ms": prove_c_ms,
            "reps": OPEN_REPS, "proof_bytes": len(blob),
            "open_l0_ms": l0_ms, "open_l0_ms_min": l0_min, "config": OPEN_CONFIG_TEXT}
    # proof-of-work search alone: hashes scanned >= smallest nonce + 1
    pw = []
    for seed in range(3):
        prefix = bytes([seed]) * 16
        t0 = time.perf_counter()
        n = bz.pow_first_nonce(prefix, 24, ctx=ctx)
        pw.append((n + 1) / (time.perf_counter() - t0))
    info["pow_24bit_hashes_per_s_lower_bound"] = float(np.median(pw))
    pd.free()
    b.free()
    info["bit_mle_2^20"] = _bench_bit_mle(ctx, bz)
    return info


OPEN_REPS = 20   # timed repetitions of every opening call (after one warm-up)
BIT_MLE_CONFIG = dict(initial_k=10, recursive_ks=[5], log_inv_rates=[2, 2], queries=[148, 64],
                      grinding_bits=[16, 8], fold_grinding_bits=[0, 2], ood_samples=[0, 1],
                      hash_kind=1)
BIT_MLE_ROUND0_BITS = 8


def _bench_bit_mle(ctx, bz):
    """The 2^20-word witness (2^10 lanes x 2^10 columns, rate 1/4, ChaCha seed
    0) opened at one random point through BinaryPcs: commit, round 0 (8-bit
    grind), open_bit_mle (ring switch + open_basis + recursive Ligerito,
    BIT_MLE_CONFIG).  Host wall time per call, median of OPEN_REPS after a
    warm-up, with p99 (the slowest rep at this count)."""
    from bitz_gb300 import codec

    m = 20
    pcs = bz.BinaryPcs(m, bz.LigeritoConfig(**BIT_MLE_CONFIG), BIT_MLE_ROUND0_BITS, ctx)
    d = bz.DeviceArray.chacha(0, 1 << m, ctx)
    point = np.random.default_rng(0).integers(0, 2**64, (m + 7, 2), dtype=np.uint64)
    ts = {"commit_ms": [], "round0_ms": [], "open_bit_mle_ms": []}
    nbytes = 0
    for _ in range(OPEN_REPS + 1):
        ctx.synchronize()
        t0 = time.perf_counter()
        c, pd = pcs.commit(d)
        t = bz.Blake3Transcript()
        t.absorb_slice(c.root)
        t1 = time.perf_counter()
        r0 = pcs.prove_round0(t, d)
        t2 = time.perf_counter()
        op = pcs.open_bit_mle(t, d, pd, r0, point)
        t3 = time.perf_counter()
        w = codec.Writer()
        r0.write(w)
        op.write(w)
        nbytes = len(w.into_bytes())
        pd.free()
        del op, r0, w, t, c  # released here, not inside the next rep's timed calls
        for k, v in zip(ts, (t1 - t0, t2 - t1, t3 - t2)):
            ts[k].append(v * 1e3)
    d.free()
    out = {k: statistics.median(v[1:]) for k, v in ts.items()}
    out.update({k.replace("_ms", "_p99_ms"): max(v[1:]) for k, v in ts.items()})
    out["reps"] = OPEN_REPS
    out["proof_stream_bytes"] = nbytes
    out["config"] = "BinaryPcs round 0 (8-bit grind) + open_bit_mle, " + str(BIT_MLE_CONFIG)
    return out


class _GkrTranscript:
    """The library's host BLAKE3 transcript as the GKR prover's transcript:
    each message is absorbed, each challenge is a field challenge."""

    def __init__(self, bz):
        self.t = bz.Blake3Transcript()
        self.t.absorb(b"gkr-bench")

    def send(self, stage, msg):
        self.t.absorb(bytes([stage]) + b"".join(np.asarray(m, np.uint64).tobytes() for m in msg))

    def challenge(self, stage):
        return self.t.get_field_challenge()


def _bench_gkr(ctx, bz):
    """Forest::prove (the dense grand-product GKR over the forest's leaf grid)
    at 2^27 leaves, the reference's own 2^27-bit forest (2^17 rows x 2^10
    columns, src/bitz/forest.rs), and at 2^22: the leaf grid is built on the
    device from the packed bits and the row images, then every layer's
    rounds run on the GPU with the transcript on the host (BLAKE3, one
    absorb and one challenge per round)."""
    from bitz_gb300 import gkr as K

    out = {}
    for t, s, reps in ((12, 10, 5), (17, 10, 3)):
        rng = np.random.default_rng(77 + t)
        rows, cols = 1 << t, 1 << s
        packed = rng.integers(0, 2**64, ((cols + 63) // 64, rows), dtype=np.uint64)
        images = rng.integers(0, 2**64, (rows, 2), dtype=np.uint64)
        zeta = [rng.integers(0, 2**64, 2, dtype=np.uint64) for _ in range(s)]
        K.forest_prove(packed, images, t, s, zeta, _GkrTranscript(bz), ctx)   # warm
        ms = []
        for _ in range(reps):
            tr = _GkrTranscript(bz)
            t0 = time.perf_counter()
            K.forest_prove(packed, images, t, s, zeta, tr, ctx)
            ms.append((time.perf_counter() - t0) * 1e3)
        rounds = sum(k + 1 for k in range(s, s + t))
        out[f"2^{t + s}"] = {"ms": statistics.median(ms), "rows": rows, "cols": cols,
                             "leaves": rows * cols, "transcript_rounds": rounds,
                             "reps": reps}
    out["note"] = ("wall time of bz_gkr_forest_prove through the Python API: leaf grid upload "
                   "and build, product layers, every round's kernels and the mailbox post of "
                   "its two sums, the host transcript called back into Python once per round")
    return out


def _geometric_sizes(rng, n, lo=14, hi=26, q=0.97):
    ks = np.arange(lo, hi + 1)
    w = q ** (ks - lo)
    w /= w.sum()
    return rng.choice(ks, size=n, p=w)


def _bench_plain_mix(ctx, bz, L, _lib, hp, sizes, params):
    """The plain one-at-a-time GPU path over a request list: per request a
    synchronous bz_commit of its host message (H2D inside), its opened rows
    and multi-proof at positions [0, 1, 7], then free.  Returns (elements per
    second, {log2 size: median per-request ms})."""
    import ctypes

    pos = np.array([0, 1, 7], np.uint64)
    per_size = {}
    total = 0
    ctx.synchronize()
    t0 = time.perf_counter()
    for k in sizes:
        k = int(k)
        p = params[k]
        pc = p.to_c()
        t1 = time.perf_counter()
        h = ctypes.c_void_p()
        root = (ctypes.c_uint8 * 32)()
        _lib.check(ctx.handle, L.bz_commit(ctx.handle, hp, 1 << k, ctypes.byref(pc),
                                           ctypes.byref(h), root))
        rows = np.empty((3, p.num_ntts(), 2), np.uint64)
        _lib.check(ctx.handle, L.bz_commitment_rows(h, _lib.ptr(pos), 3, _lib.ptr(rows)))
        depth = p.k_code()
        proof = np.empty((3 * depth, 32), np.uint8)
        n = ctypes.c_size_t()
        _lib.check(ctx.handle, L.bz_commitment_multiproof(h, _lib.ptr(pos), 3, _lib.ptr(proof),
                                                          3 * depth, ctypes.byref(n)))
        L.bz_commitment_free(h)
        per_size.setdefault(k, []).append((time.perf_counter() - t1) * 1e3)
        total += 1 << k
    wall = time.perf_counter() - t0
    return total / wall, {k: statistics.median(v) for k, v in per_size.items()}


def _bench_serve(ctx, bz, args, plain_rate=None):
    """Poisson commit-then-open requests with log2 sizes from a truncated
    geometric on [14, 26], admitted by free HBM (continuous batching); the
    arrival rate is swept to saturation.  Each request is one
    ``submit_commit_open`` of a host message (the server queues the opening,
    rows + multi-proof at 3 positions, when the commit completes) and the
    request loop reacts to the server's completion queue.

    The baseline is the plain one-at-a-time GPU path on the same mix: the
    same kind of request list served by synchronous bz_commit + rows +
    multi-proof calls (``plain_same_mix``).  Offered loads are fractions of
    that plain rate, so load 1.0 is what the plain path can just sustain.
    Besides throughput and p50/p99 submit-to-opened latency, each rate
    reports the slowdown: a request's latency over the plain path's median
    latency for a request of its size (sizes span 2^14 to 2^26, so raw
    latency percentiles mostly reflect the size mix).  The saturating point
    (1.5 x) serves ``--serve-requests`` requests (10k by default); the lighter
    loads a tenth of that."""
    import numpy as np
    from bitz_gb300 import serve as S

    rng = np.random.default_rng(4)
    # pinned host messages: one buffer of the largest size, prefixes reused
    import ctypes

    from bitz_gb300 import _lib

    L = _lib.lib()
    max_n = 1 << 26
    hp = ctypes.c_void_p()
    _lib.check(None, L.bz_host_alloc_pinned(16 * max_n, ctypes.byref(hp)))
    _lib.check(None, L.bz_chacha_fill_host(4, 0, hp, max_n, os.cpu_count() or 1))
    params = {k: bz.PcsParams(k + 7, 2, k // 2, 1) for k in range(14, 27)}
    # warm every shape once (twiddles, schedules), then the plain baseline
    _bench_plain_mix(ctx, bz, L, _lib, hp, list(range(14, 27)), params)
    plain_sizes = _geometric_sizes(np.random.default_rng(5), max(args.serve_requests // 5, 200))
    plain, solo_ms = _bench_plain_mix(ctx, bz, L, _lib, hp, plain_sizes, params)
    _, solo_all = _bench_plain_mix(ctx, bz, L, _lib, hp, list(range(14, 27)) * 3, params)
    for k, v in solo_all.items():
        solo_ms.setdefault(k, v)
    base = plain
    out = {"requests_at_saturation": args.serve_requests, "unit": UNIT,
           "sizes": "truncated geometric on [14,26], q=0.97",
           "plain_same_mix": plain,
           "plain_same_mix_requests": len(plain_sizes),
           "plain_same_mix_path": "one request at a time: bz_commit (host message, H2D inside) "
                                  "+ bz_commitment_rows + bz_commitment_multiproof at 3 positions",
           "load_reference": base, "c4_mix_plain_device_rate": plain_rate,
           "solo_ms_by_log2_size": {str(k): v for k, v in sorted(solo_ms.items())},
           "rates": []}
    # one long-running server for every load point, warmed up first: its
    # stream-ordered pool grows to hold several of the largest requests at
    # once, as a server that has been running would have
    srv = S.Server(ctx, n_slots=6)
    srv.next_done(0, 0)                                   # start the completion queue
    warm = [srv.submit_commit_open_ptr(hp.value, 1 << k, params[k], [0, 1, 7])
            for k in (26, 26, 26, 26, 25, 24, 20, 16)]
    for rid in warm:
        srv.wait(rid, S.OPENED, 120000)
        srv.release(rid)
    srv.next_done(1 << 12, 0)                             # drop the warm-up's completions
    for load in (0.3, 0.6, 0.9, 1.5):
        n_req = args.serve_requests if load >= 1.0 else max(args.serve_requests // 10, 50)
        sizes = _geometric_sizes(rng, n_req)
        total_elems = int(sum(1 << int(k) for k in sizes))
        lam = load * base / (total_elems / n_req)        # requests per second
        arrivals = np.cumsum(rng.exponential(1.0 / lam, n_req))
        lat, slow = [], []
        rid_size = {}
        t0 = time.perf_counter()
        i = done = 0
        while done < n_req:
            now = time.perf_counter() - t0
            while i < n_req and arrivals[i] <= now:
                k = int(sizes[i])
                rid = srv.submit_commit_open_ptr(hp.value, 1 << k, params[k], [0, 1, 7])
                rid_size[rid] = k
                i += 1
            if i < n_req:
                wait_us = int(max(0.0, arrivals[i] - (time.perf_counter() - t0)) * 1e6)
            else:
                wait_us = 20000
            for rid, st in srv.next_done(256, wait_us):
                if st == S.OPENED:
                    t = srv.times(rid)
                    ms = (t[4] - t[0]) / 1e6
                    lat.append(ms)
                    slow.append(ms / solo_ms[rid_size.pop(rid)])
                    srv.release(rid)
                    done += 1
                elif st == S.FAILED:
                    raise RuntimeError("serving request failed")
        wall = time.perf_counter() - t0
        srv.next_done(1 << 12, 0)
        lat.sort()
        slow.sort()
        q = lambda a, f: a[min(len(a) - 1, int(f * len(a)))]
        out["rates"].append({
            "offered_load": load, "requests": n_req, "log2_size_mean": float(sizes.mean()),
            "arrival_rate_per_s": lam, "throughput": total_elems / wall,
            "throughput_vs_plain_same_mix": total_elems / wall / plain,
            "p50_ms": q(lat, 0.5), "p99_ms": q(lat, 0.99),
            "slowdown_p50": q(slow, 0.5), "slowdown_p99": q(slow, 0.99),
            "wall_s": wall})
    srv.close()
    out["server"] = {"slots": 6, "policy": "smallest first, 500 ms aging bound; requests of "
                                             "<= 2^20 elements on the 3 high-priority slots"}
    L.bz_host_free_pinned(hp)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--skip-shapes", action="store_true")
    ap.add_argument("--skip-open", action="store_true")
    ap.add_argument("--skip-gkr", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--schedule", default=None,
                    help="fixed NTT schedule for the headline shape (e.g. 0x1002) instead of "
                         "autotuning; profiling runs use the schedule a default run picked")
    ap.add_argument("--only-commit", action="store_true",
                    help="time the device commit loop only (profiling runs)")
    ap.add_argument("--only-open", action="store_true",
                    help="the device commit loop and the opening leg only (profiling runs)")
    ap.add_argument("--log-n", type=int, default=None, help="override log2 elements")
    ap.add_argument("--serve-requests", type=int, default=10000,
                    help="requests per offered-load point of the serving sweep")
    args = ap.parse_args()
    if args.log_n is not None:
        global LOG_N, LOG_LANES, MSG_BYTES
        LOG_N = args.log_n
        LOG_LANES = args.log_n // 2
        MSG_BYTES = 16 << LOG_N
    ws, rank, local = _dist()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
