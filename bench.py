#!/usr/bin/env python
"""Benchmark of the effective-Hamiltonian hot path on one GB300.

Workload (the configuration the headline metric is quoted at, D = 2048): two-site DMRG
on the spin-1/2 J1-J2 Heisenberg model (J1 = 1, J2 = 0.5) on a width-6 cylinder of
length 24, snake-ordered into a 144-site chain, MPO from the channel-assignment builder
with charge-definite channels, Float64, U(1) symmetric (total Sz = 0) seeded random
initial MPS at D = 2048 (`--symmetry none`: dense, no symmetry), split-precision (bf16x3)
contractions with FP64 Lanczos / gauge.

One step = one DMRG2 local update (dmrg.jl:211-244) at the central bond -- H_eff build
and prepare, the Galerkin matvec, the adaptive Lanczos eigensolve, the truncated
(per-charge-block) factorisation -- plus the environment step the next bond of a sweep
needs.

value  = H_eff algorithmic flops per second of step time (TFLOP/s); algorithmic = the
         nonzero scalar products of the block-sparse contractions (counted on one matvec);
e2e    = the same, driven through the C ABI with host buffers (x0 uploaded from pinned
         host memory, the new AL / S / AR downloaded every step);
roofline = the persistent tcgen05 split GEMM (dominant contraction kernel), timed with
         CUDA events on the library's stream, against the measured sustained BF16 peak;
fp64_gpu = the plain FP64 GPU path on the same bond.

`--workload vumps-sweep` times a different configuration: 64 independent TFIM chains
(one-site VUMPS, g in [0.1, 2.0], D in {64, 128, 192, 256}) solved concurrently.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "mpskit.jl_gb300"), ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "DMRG sweep s & H_eff TFLOP/s at D=2048, split-prec vs FP64 GPU at |ΔE/E|≤1e-9"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--D", type=int, default=2048)
    ap.add_argument("--Lx", type=int, default=24)
    ap.add_argument("--Ly", type=int, default=6)
    ap.add_argument("--precision", default="bf16x3", choices=["bf16x3", "tf32x3", "fp64"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--trace", action="store_true",
                    help="after the timed steps, trace one more step: time per issuing "
                         "source site (gb_ctx_trace_begin/end)")
    ap.add_argument("--seed", type=int, default=1234 + 5)
    ap.add_argument("--svd", default="gram", choices=["gesvd", "gesvdp", "gram"])
    ap.add_argument("--eig", default="syevd", choices=["syevd", "syevj", "syevd32"],
                    help="eigensolver of the Gram factorisations")
    ap.add_argument("--lanes", type=int, default=8, help="host-thread lanes of the gauge step")
    ap.add_argument("--symmetry", default="u1", choices=["u1", "none"],
                    help="u1: U(1) (total Sz = 0) block-sparse state and MPO; none: dense")
    ap.add_argument("--workload", default="dmrg2",
                    choices=["dmrg2", "dmrg2-sweep", "matvec", "vumps-sweep", "vumps-xxz",
                             "grassmann"],
                    help="dmrg2: the headline DMRG2 step; dmrg2-sweep: full DMRG2 sweeps of "
                         "the same state (checkpointed environments); matvec: repeated H_eff "
                         "applications at the central bond (a small case for profiling); "
                         "vumps-sweep: 64 "
                         "independent TFIM "
                         "chains (VUMPS, g in [0.1, 2], D in {64..256}) solved concurrently; "
                         "vumps-xxz: one-site VUMPS of the XXZ chain (Jz = 1.5, sublattice-"
                         "rotated) at D = 256, "
                         "plain FP64 against the split precision; grassmann: GradientGrassmann "
                         "cost+gradient evaluations on a finite TFIM chain (L=64, D=128)")
    ap.add_argument("--schedule", default="grouped",
                    choices=["grouped", "persistent", "persistent_dense", "tile"],
                    help="split GEMM schedule: grouped (one launch per contraction over its "
                         "U(1) charge blocks; the default) or the dense-embedding schedules")
    ap.add_argument("--tile-n", type=int, default=0, choices=[0, 128, 256],
                    help="output tile width of the split GEMM (0: chosen per GEMM shape)")
    ap.add_argument("--window", type=int, default=8,
                    help="bonds of the measured sweep window (split and plain FP64 from the "
                         "same state); 0 skips it")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the split-vs-FP64 eigensolve comparison at the bench bond")
    ap.add_argument("--sweeps", type=int, default=1, help="sweeps of --workload dmrg2-sweep")
    ap.add_argument("--describe", action="store_true",
                    help="--workload matvec: print the operator's contraction steps and plans")
    ap.add_argument("--env-storage", default="packed", choices=["packed", "checkpoint"],
                    help="dmrg2-sweep: every environment resident tile-packed, or every "
                         "--checkpoint-th one dense with recomputation")
    ap.add_argument("--checkpoint", type=int, default=12,
                    help="dmrg2-sweep: environments kept resident every this many sites")
    ap.add_argument("--ref-budget", type=float, default=90.0,
                    help="seconds of timed CPU steps in --impl reference (bounded sample)")
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--vumps-iters", type=int, default=6)
    return ap.parse_args()


_T0 = time.perf_counter()


def log(msg):
    print(f"[bench {time.perf_counter() - _T0:8.1f}s] {msg}", file=sys.stderr, flush=True)


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], [], set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 7:
                    continue
                try:
                    sm.append(float(f[0]))
                    mx.append(float(f[1]))
                except ValueError:
                    continue
                for n, v in zip(names, f[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except Exception:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allsum(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- oracle timing (CPU)

def oracle_threads():
    try:
        from threadpoolctl import threadpool_info
        return max([i.get("num_threads", 1) for i in threadpool_info()] + [1])
    except Exception:
        return os.cpu_count() or 1


def run_reference(args):
    """--impl reference: the same workload on the host cores with the oracle's block-sparse
    U(1) restatement (oracle/blocksparse.py: TensorKit-style blockwise contractions), from
    the same seeded state: blockwise canonical form, environments to the central bond, then
    per step one DMRG2 local update at that bond (Galerkin matvec, adaptive Lanczos on the
    charge-allowed entries, blockwise truncated SVD) plus the environment step the next bond
    needs.  H_eff flops are counted as in the GPU arm: 2 x the multiply-adds of the charge
    blocks of every contraction.  The CPU needs no warm-up beyond one step; timed steps stop
    after --ref-budget seconds (a bounded sample of the requested steps)."""
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        return
    import mpsgb
    from mpsgb.operators import SPIN_HALF_CHARGES as QP
    from oracle import blocksparse as B
    from oracle import mps as P
    if args.symmetry != "u1":
        print(json.dumps({"impl": "reference", "unavailable":
                          "the CPU arm restates the U(1) workload only"}), flush=True)
        return
    t_setup = time.perf_counter()
    H = mpsgb.j1j2_cylinder(args.Lx, args.Ly, dtype=np.float64, u1=True)
    n = len(H)
    pos = n // 2 - 1
    D = args.D
    As, qb = mpsgb.u1.random_u1_tensors(n, D, args.seed, 0, np.float64)
    psi = B.canonical_u1(As, qb, QP, pos + 1)
    del As
    log("reference: canonical form done")
    envs = B.FiniteEnvironmentsU1(psi, H, keep_newest=True)
    envs.leftenv(pos, psi)
    envs.rightenv(pos + 1, psi)
    t_setup = time.perf_counter() - t_setup
    log(f"reference: environments at bond {pos} done ({t_setup:.1f} s setup)")
    alg = P.DMRG2(maxdim=D, cutoff=1e-10)
    state = {"eps_local": 1.0, "eps_trunc": 0.0, "decay": 0.0}

    def step(stats):
        el, et, dec, val = B.dmrg2_local_update(pos, False, psi, H, alg, envs, state["eps_local"],
                                                state["eps_trunc"], state["decay"], stats)
        state.update(eps_local=el, eps_trunc=et, decay=dec, val=val)
        A = psi.AR[pos + 1]
        B.transfer_right(envs.rightenv(pos + 1, psi), H.W[pos + 1], A, psi.qb[pos + 1], QP,
                         psi.qb[pos + 2], envs.dq[pos + 1])

    for i in range(min(args.warmup, 1)):
        step({"matvecs": 0})
        log(f"reference: warm-up step {i} done")
    stats = {"matvecs": 0}
    ts = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        step(stats)
        ts.append(time.perf_counter() - t0)
        log(f"reference: step {i}: {ts[-1]:.2f} s")
        if sum(ts) > args.ref_budget:
            break
    tot = sum(ts)
    value = stats["block_flops"] / tot / 1e12
    threads = oracle_threads()
    sample = (f"{len(ts)} of the {args.steps} requested steps (timed steps stop after {args.ref_budget:.0f} s);"
              f" one step = DMRG2 local update at bond {pos} + environment step, oracle "
              f"block-sparse (numpy/BLAS, {threads} threads), {stats['matvecs'] / len(ts):.1f} "
              f"matvecs per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": len(ts), "warmup": min(args.warmup, 1),
        "ms_per_step": 1e3 * tot / len(ts), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"J1-J2 Heisenberg {args.Ly}x{args.Lx} cylinder ({n} sites), DMRG2 "
                               f"local update + env step at bond {pos}, D={D}, Float64, U(1) "
                               f"total Sz = 0, block-sparse", "symmetry": "u1", "D": D, "L": n,
                   "mpo_width_at_bond": int(H.W[pos].shape[3]), "sample": sample,
                   "setup_s": t_setup},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "local_energy": state.get("val"),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm

def run_ours(args):
    world, rank, local, pg = dist_setup(args)
    import mpsgb
    from mpsgb.algorithms import SweepStats, dmrg2_local_update

    ctx = mpsgb.context(local)
    prec = args.precision
    ctx.set_precision(prec)
    ctx.set_svd_method(args.svd)
    ctx.set_gauge(args.eig, args.lanes)
    ctx.set_gemm_schedule(args.schedule, args.tile_n)
    backend = mpsgb.GB300Backend(prec, local)
    u1 = args.symmetry == "u1"
    H = mpsgb.j1j2_cylinder(args.Lx, args.Ly, dtype=np.float64, u1=u1)
    n = len(H)
    pos = n // 2 - 1
    D = args.D
    t_setup = time.perf_counter()
    charges = None
    if u1:
        As, qb = mpsgb.u1.random_u1_tensors(n, D, args.seed + rank, 0, np.float64)
        charges = (qb, mpsgb.operators.SPIN_HALF_CHARGES)
    else:
        As = mpsgb.states.random_tensors(n, 2, D, args.seed + rank, np.float64)
    log(f"random tensors ready (L={n}, D={D}, symmetry {args.symmetry})")
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=charges)
    del As
    ctx.synchronize()
    log("canonical MPS built on the device")
    # the right environments of the measured window stay resident (2 GB each at D = 2048)
    envs = mpsgb.FiniteEnvironments(psi, H, resident=False, keep_left={pos},
                                    keep_right=set(range(pos + 1, pos + args.window + 2)))
    envs.precision = backend.code
    envs.leftenv(pos, psi)
    ctx.synchronize()
    log("left environments built")
    envs.rightenv(pos + 1, psi)
    ctx.synchronize()
    log(f"right environments built; device status {ctx.device_status()}")
    t_setup = time.perf_counter() - t_setup
    alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-10, backend=backend)
    state = {"eps_local": 1.0, "eps_trunc": 0.0, "decay": 0.0}

    from mpsgb import _lib as L
    Wd = H.device(ctx, np.float64)
    GR_next = mpsgb.DeviceTensor(ctx, L.GB_KIND_GR, np.float64,
                                 (psi.AR[pos + 1].dims[0], Wd[pos + 1].dims[0], psi.AR[pos + 1].dims[0]))

    def step(stats):
        el, et, dec, val = dmrg2_local_update(pos, False, psi, H, alg, envs, state["eps_local"],
                                              state["eps_trunc"], state["decay"], stats)
        state.update(eps_local=el, eps_trunc=et, decay=dec, val=val)
        # environment step the next bond of a left-moving sweep needs: GR[pos] from the new
        # AR[pos+1]; written to a side buffer so that GR[pos+1] stays cached for the next step
        t0 = time.perf_counter()
        A = psi.AR[pos + 1]
        nonlocal GR_next
        want = (A.dims[0], Wd[pos + 1].dims[0], A.dims[0])
        if GR_next.dims != want:
            GR_next = mpsgb.DeviceTensor(ctx, L.GB_KIND_GR, np.float64, want)
        L.check(L.lib().gb_env_transfer_right(ctx.handle, envs.rightenv(pos + 1, psi).handle,
                                              Wd[pos + 1].handle, A.handle, A.handle,
                                              backend.code, GR_next.handle))
        if stats.sync:
            ctx.synchronize()
        stats.t["env"] += time.perf_counter() - t0

    warm = SweepStats(sync=True)
    for i in range(args.warmup):
        step(warm)
        ctx.synchronize()
        log(f"warmup step {i}: matvecs {warm.matvecs} phases {warm.t}")
    ctx.synchronize()
    stats = SweepStats(sync=True)
    launches0 = ctx.kernel_launches()
    barrier(pg)
    ctx.synchronize()
    try:
        import torch
        nvtx = torch.cuda.nvtx
    except Exception:
        nvtx = None
    ctx.read_work(reset=True)
    with ClockSampler(local) as clocks:
        if nvtx:
            nvtx.range_push("timed")
        ctx.profile_begin()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step(stats)
        ctx.synchronize()
        t_wall = time.perf_counter() - t0
        prof = ctx.profile_end()
        if nvtx:
            nvtx.range_pop()
    barrier(pg)
    launches = ctx.kernel_launches() - launches0
    tile_flops_timed = ctx.read_work(reset=True)["tile_flops"]
    t_dev = prof["region_ms"] / 1e3          # CUDA-event time of the region on the stream
    t_step = max(t_wall, t_dev)
    t_max = allmax(pg, t_step)
    ms_per_step = 1e3 * t_max / args.steps
    # flop accounting (untimed): one H_eff matvec at the same bond -- the charge-block flops
    # of its contractions (2 sum_g M_g N_g K_g over the blocks of every GEMM, the work a
    # blockwise library does; the dense GEMM count without symmetry), the nonzero products
    # (sum_k nnz(A[:, k]) nnz(B[k, :])) and the tile work the tensor pipe executes
    count = heff_count_pass(ctx, psi, H, envs, backend, pos, u1) if prec != "fp64" else None
    trace = None
    if args.trace:
        # one more (untimed) step under the launch trace: time per issuing source site
        ctx.trace_begin()
        tstats = SweepStats(sync=True)
        step(tstats)
        span, sites = ctx.trace_end()
        trace = {"span_ms": span, "matvecs": tstats.matvecs,
                 "sites": [[nm, round(ms, 3), ev] for nm, ms, ev in sites[:24]]}
        log(f"launch trace: {span:.1f} ms over {sum(ev for _, _, ev in sites)} events")
        for nm, ms, ev in sites[:24]:
            log(f"  {nm:28s} {ms:9.3f} ms {ev:6d} events")
    if count:
        heff_alg = count["block_flops"] * stats.matvecs
        rho = count["nonzero_flops"] / max(1.0, count["tile_flops"])
    else:
        heff_alg, rho = stats.heff_flops, 1.0
    value = allsum(pg, heff_alg) / t_max / 1e12

    pk = peaks() or {}
    peak_bf16 = pk.get("bf16_tflops_sustained")
    peak_src = "measured (sustained)" if peak_bf16 else "fallback"
    peak_bf16 = peak_bf16 or 1700.0
    split = 1.0 if prec == "fp64" else 3.0
    grouped = prof["grouped"]["launches"] > 0
    if grouped:
        # the grouped sector-block GEMM: its charge-block flops over its own kernel time
        kms = prof["grouped"]["ms"]
        gemm_alg = prof["grouped"]["flops"] / (kms / 1e3) / 1e12 if kms > 0 else 0.0
        kernel, klaunch = "gemm_grouped_kernel", prof["grouped"]["launches"]
    else:
        # the dense-embedding GEMM: executed tile work x (nonzero / tile) of the counted
        # matvec (the dense case has rho ~ 1, below 1 only by partial-tile padding)
        kms = prof["persistent"]["ms"]
        gemm_alg = rho * tile_flops_timed / (kms / 1e3) / 1e12 if kms > 0 else 0.0
        kernel, klaunch = "gemm_bf16x3_persistent", prof["persistent"]["launches"]
    achieved = split * gemm_alg
    roofline = {
        "bound": "tensor", "kernel": kernel, "achieved": achieved,
        "peak": peak_bf16, "unit": "TFLOP/s", "frac": achieved / peak_bf16,
        "peak_source": peak_src, "algorithmic_tflops": gemm_alg,
        "executed_tile_tflops_per_product": tile_flops_timed / max(prof["gemm_ms"] / 1e3, 1e-12) / 1e12,
        "launches": klaunch, "kernel_ms": kms,
        "kernel_share_of_step": kms / max(1e-9, prof["region_ms"]),
        "other_split_gemm": {"kernel": "gemm_bf16x3_persistent (environment step)",
                             "ms": prof["persistent"]["ms"],
                             "launches": prof["persistent"]["launches"]} if grouped else None,
        "traffic": None,
    }
    if (grouped and u1 and prec == "bf16x3" and D == 2048 and args.Lx == 24 and args.Ly == 6
            and args.seed == 1234 + 5):
        # DRAM bytes (read + write) per grouped launch of this workload's AC2 matvec, from the
        # ncu capture summarised in profiles/gemm_grouped_D2048_u1_dram.txt (the three
        # launches of one matvec: 298.5 + 574.8 + 46.5 MB)
        roofline["traffic"] = 306.6e6
        roofline["traffic_source"] = "profiles/gemm_grouped_D2048_u1_dram.txt"

    # ---------------- end to end through the C ABI with host buffers
    log(f"timed region done: {t_wall:.3f}s wall, {t_dev:.3f}s device; status {ctx.device_status()}")
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, ctx, psi, H, envs, alg, pos, state, pg,
                      count["block_flops"] if count else None)
        log("e2e done")

    accuracy = None
    if prec != "fp64" and not args.no_accuracy:
        accuracy = accuracy_compare(ctx, psi, H, envs, backend, pos)
        log(f"accuracy at bond {pos}: {accuracy}")
    window = None
    if prec != "fp64" and not args.no_fp64_compare and args.window > 0:
        window = window_compare(ctx, psi, H, envs, pos, args.window, prec, D, state)
        log(f"window of {args.window} bonds: split {window['split']['s_per_bond']:.3f} s/bond, "
            f"fp64 {window['fp64']['s_per_bond']:.3f} s/bond")

    cpu = None
    if not args.no_cpu_baseline and rank == 0 and world == 1 and u1:
        cpu = cpu_baseline_sample(psi, H, envs, pos, stats.matvecs / args.steps)
        log(f"cpu baseline done: {cpu['value']:.4f} TFLOP/s")

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == "fp64" else f"f64 ({prec} split contractions)",
            "data": "synthetic",
            "config": {
                "workload": f"J1-J2 Heisenberg {args.Ly}x{args.Lx} cylinder ({n} sites), DMRG2 "
                            f"local update + env step at bond {pos}, D={D}, Float64, "
                            + ("U(1) total Sz = 0, block-sparse" if u1 else "dense, no symmetry"),
                "symmetry": args.symmetry,
                "model": "J1=1, J2=0.5, snake order", "D": D, "L": n,
                "mpo_width_at_bond": int(H.W[pos].shape[3]), "precision": prec,
                "svd": args.svd, "eig": args.eig, "lanes": args.lanes,
                "tile_n": args.tile_n or "per shape",
                "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (GL/GR/T1 >> 129 MB)",
            },
            "gpu_launches": launches,
            "heff_flops_per_step": heff_alg / args.steps,
            "heff_flops_per_matvec": {
                "nonzero_products": count["nonzero_flops"] if count else None,
                "tile_executed_per_product": count["tile_flops"] if count else None,
                "dense_equivalent": stats.heff_flops / max(1, stats.matvecs)},
            "matvecs_per_step": stats.matvecs / args.steps,
            "phase_s_per_step": {k: v / args.steps for k, v in stats.t.items()},
            "local_energy": state.get("val"), "eps_trunc": state.get("eps_trunc"),
            "setup_s": t_setup,
            "roofline": roofline,
            "launch_trace": trace,
            "accuracy_vs_fp64": accuracy,
            "sweep_window": window,
            "clocks": clocks.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def heff_count_pass(ctx, psi, H, envs, backend, pos, u1):
    """One AC2 matvec with the GEMM work counters on: charge-block flops (the grouped GEMMs'
    2 sum_g M_g N_g K_g; without symmetry the dense GEMM flops), nonzero-product flops and
    tile flops executed per split product."""
    import mpsgb
    ctx.read_work(reset=True)
    ctx.set_counting(True)
    try:
        Heff = mpsgb.AC2_hamiltonian(pos, psi, H, envs, backend)
        x = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
        Heff.set_sectors(x)
        ctx.synchronize()
        ctx.read_work(reset=True)
        ctx.profile_begin()
        Heff(x)
        prof = ctx.profile_end()
        out = ctx.read_work(reset=True)
    finally:
        ctx.set_counting(False)
    if prof["grouped"]["launches"] > 0:
        out["block_flops"] = prof["grouped"]["flops"]
    else:
        out["block_flops"] = out["nonzero_flops"] if u1 else prof["gemm_flops"]
    return out


def cpu_baseline_sample(psi, H, envs, pos, matvecs):
    """The oracle's block-sparse operator (oracle/blocksparse.py) on the host cores, on the
    environments and state of the GPU run at the bench bond: the operator build plus as many
    matvecs as one GPU local update took (a bounded sample of one local update; the block SVD
    is left out).  Rate = charge-block flops / time, as in the GPU arm."""
    from mpsgb.operators import SPIN_HALF_CHARGES as QP
    from oracle import blocksparse as B
    GL = envs.leftenv(pos, psi).numpy()
    GR = envs.rightenv(pos + 1, psi).numpy()
    x = __import__("mpsgb").ac2_from(psi.AL[pos], psi.ac(pos + 1))
    ql, _, qr, _ = x.charges
    x = x.numpy()
    dq = B.mpo_channel_charges([H.W[i] for i in range(len(H))], QP)
    k = max(1, int(round(matvecs)))
    t0 = time.perf_counter()
    op = B.JordanAC2U1(GL, H.W[pos], H.W[pos + 1], GR, ql, QP, qr, dq[pos], dq[pos + 2])
    t_build = time.perf_counter() - t0
    for _ in range(k):
        x = op(x)
        x /= np.linalg.norm(x)
    t = time.perf_counter() - t0
    threads = oracle_threads()
    return {"value": op.block_flops() * k / t / 1e12, "unit": "TFLOP/s", "cores": threads,
            "kind": "port",
            "sample": f"oracle block-sparse JordanAC2 at bond {pos} on the device-built "
                      f"environments: operator build ({t_build:.1f} s) + {k} matvecs (the "
                      f"matvec count of one GPU local update), {t:.1f} s; numpy/BLAS with "
                      f"{threads} threads; the block SVD and the environment step left out"}


def accuracy_compare(ctx, psi, H, envs, backend, pos, fp64_maxiter=8):
    """The precision condition of the metric at the bench bond: from the same state,
    environments and start vector, the split-precision Lanczos solve followed by its FP64
    refinement step (one FP64 matvec: Rayleigh quotient and residual of the split solution
    with the FP64 operator) against the FP64 Lanczos solve of the same local problem."""
    import mpsgb
    fp64 = mpsgb.GB300Backend("fp64", backend.device)
    x0 = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    H64 = mpsgb.AC2_hamiltonian(pos, psi, H, envs, fp64)
    Hs = mpsgb.AC2_hamiltonian(pos, psi, H, envs, backend)

    def refine(x):
        y = H64(x)
        nx2 = x.dot(x).real
        e = float(np.real(x.dot(y))) / nx2
        y.axpy_(-e, x)
        return e, y.norm() / np.sqrt(nx2)

    out = {}
    for label, op, tol, mi in (("split", Hs, 1e-10, 12), ("fp64", H64, 1e-11, fp64_maxiter)):
        ctx.synchronize()
        t0 = time.perf_counter()
        lam, x, info = mpsgb.fixedpoint(op, x0, "SR", mpsgb.Lanczos(krylovdim=30, maxiter=mi,
                                                                   tol=tol, eager=False))
        ctx.synchronize()
        t = time.perf_counter() - t0
        e, r = refine(x)
        out[label] = {"eigsolve_s": t, "matvecs": info.numops, "converged": info.converged,
                      "ritz_value": lam, "energy_fp64": e, "residual_fp64": r}
    e_s, e_d = out["split"]["energy_fp64"], out["fp64"]["energy_fp64"]
    out["delta_e_rel"] = abs(e_s - e_d) / abs(e_d)
    out["ritz_delta_rel"] = abs(out["split"]["ritz_value"] - e_d) / abs(e_d)
    out["how"] = ("same bond, state, environments and x0; split Lanczos (tol 1e-10, stops at "
                  "its noise floor) then one FP64 matvec: energy = FP64 Rayleigh quotient, "
                  "residual = |H x - E x| / |x| with the FP64 operator; against the FP64 "
                  "Lanczos solve (tol 1e-11)")
    return out


def window_compare(ctx, psi, H, envs, pos, nb, prec, D, state):
    """A sweep window measured in both precisions from the same state: `nb` consecutive
    two-site updates moving right from the bench bond (local update + the left environment
    the next bond needs), split precision first, then plain FP64 from the restored state.
    Per bond: Ritz value, matvecs; per window: seconds (device-synchronised)."""
    import mpsgb
    from mpsgb.algorithms import SweepStats, dmrg2_local_update
    sites = range(pos, pos + nb + 2)
    saved = ({i: psi.AL[i] for i in sites}, {i: psi.AR[i] for i in sites},
             {i: psi.C[i] for i in sites}, psi.center)

    def restore():
        for i in sites:
            psi.AL[i], psi.AR[i], psi.C[i] = saved[0][i], saved[1][i], saved[2][i]
        psi.center = saved[3]

    res = {}
    for label, p in (("split", prec), ("fp64", "fp64")):
        restore()
        be = mpsgb.GB300Backend(p)
        envs.precision = be.code
        alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-10, backend=be)
        envs.leftenv(pos, psi)
        envs.rightenv(pos + 1, psi)
        ctx.synchronize()
        stats = SweepStats(sync=True)
        ritz, et, dec = [], state["eps_trunc"], state["decay"]
        t0 = time.perf_counter()
        for k in range(nb):
            el, et, dec, val = dmrg2_local_update(pos + k, True, psi, H, alg, envs,
                                                  state["eps_local"], et, dec, stats)
            envs.leftenv(pos + k + 1, psi)  # the next bond's left environment
            ritz.append(val)
        ctx.synchronize()
        t = time.perf_counter() - t0
        res[label] = {"seconds": t, "s_per_bond": t / nb, "matvecs": stats.matvecs,
                      "phase_s": {k: v for k, v in stats.t.items()}, "ritz_values": ritz}
    restore()
    envs.precision = mpsgb.GB300Backend(prec).code
    res["bonds"] = [pos, pos + nb - 1]
    res["split_speedup_per_bond"] = res["fp64"]["s_per_bond"] / res["split"]["s_per_bond"]
    res["max_ritz_delta_rel"] = max(abs(a - b) / abs(b) for a, b in
                                    zip(res["split"]["ritz_values"], res["fp64"]["ritz_values"]))
    res["how"] = ("measured: the same right-moving window of two-site updates run in split "
                  "precision and in plain FP64 from the same state, each with its own Krylov "
                  "budget (AdaptiveKrylov), SVD truncation and left-environment steps; Ritz "
                  "values are those of each precision's own operator")
    return res


def run_e2e(args, ctx, psi, H, envs, alg, pos, state, pg, flops_per_matvec=None):
    """Local updates driven through the C ABI with host buffers: x0 uploaded from pinned
    host memory, eigensolve + truncated SVD on the device, AL/S/AR downloaded."""
    import ctypes

    import mpsgb
    from mpsgb import _lib as L
    try:
        import torch
        pin = lambda shape: torch.empty(int(np.prod(shape)), dtype=torch.float64, pin_memory=True)
        host_ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    except Exception:
        pin = lambda shape: np.empty(int(np.prod(shape)))
        host_ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    ac2 = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    x_host = pin(ac2.dims)
    L.check(L.lib().gb_tensor_download(ac2.handle, host_ptr(x_host), ac2.size * 8))
    Heff = mpsgb.AC2_hamiltonian(pos, psi, H, envs, alg.backend)
    # U(1): the vectors' sectors, as a C-ABI caller passes them after gb_heff_build
    # (gb_heff_set_sectors; a no-op for dense vectors)
    Heff.set_sectors(ac2)
    flops = flops_per_matvec or Heff.flops
    outs = {}

    def one():
        x = mpsgb.DeviceTensor(ctx, L.GB_KIND_AC2, np.float64, ac2.dims, charges=ac2.charges)
        L.check(L.lib().gb_tensor_upload(x.handle, host_ptr(x_host), x.size * 8))
        solver = alg.alg_eigsolve.adapt(state["decay"], state["eps_local"], state["eps_local"],
                                        state["eps_trunc"])
        lam = ctypes.c_double()
        ki = L.KrylovInfo()
        L.check(L.lib().gb_heff_eigsolve(Heff.handle, x.handle, solver.krylovdim, solver.maxiter,
                                         solver.tol, int(solver.eager), ctypes.byref(lam),
                                         ctypes.byref(ki)))
        al, S, ar, eps = mpsgb.svd_trunc(x, alg.maxdim, alg.cutoff, True)
        d2h = 0
        for t in (al, S, ar):
            key = t.dims
            if key not in outs:
                outs[key] = pin(t.dims)
            L.check(L.lib().gb_tensor_download(t.handle, host_ptr(outs[key]), t.size * 8))
            d2h += t.size * 8
        return ki.numops, d2h

    for _ in range(max(1, args.warmup)):
        one()
    barrier(pg)
    ctx.synchronize()
    t0 = time.perf_counter()
    nops, d2h = 0, 0
    for _ in range(args.steps):
        k, b = one()
        nops += k
        d2h = b
    ctx.synchronize()
    t = allmax(pg, time.perf_counter() - t0)
    fl = allsum(pg, flops * nops)
    return {"value": fl / t / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": ac2.size * 8,
            "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * t / args.steps,
            "path": "gb_heff_set_sectors once; gb_tensor_upload -> gb_heff_eigsolve -> "
                    "gb_svd_trunc -> gb_tensor_download"}


def run_matvec(args):
    """Repeated applications of the two-site operator at the central bond of the headline
    model (U(1), seeded random state, D = --D): the dominant contractions alone, for
    profiling at a size whose operands fit a few GB.  Reports charge-block TFLOP/s."""
    import mpsgb
    ctx = mpsgb.context(0)
    ctx.set_gemm_schedule(args.schedule, args.tile_n)
    backend = mpsgb.GB300Backend(args.precision, 0)
    H = mpsgb.j1j2_cylinder(args.Lx, args.Ly, dtype=np.float64, u1=True)
    n, D = len(H), args.D
    pos = n // 2 - 1
    As, qb = mpsgb.u1.random_u1_tensors(n, D, args.seed, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1,
                                       charges=(qb, mpsgb.operators.SPIN_HALF_CHARGES))
    envs = mpsgb.FiniteEnvironments(psi, H, resident=False)
    envs.precision = backend.code
    Heff = mpsgb.AC2_hamiltonian(pos, psi, H, envs, backend)
    x = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    Heff.set_sectors(x)
    y = Heff.new_vector()
    y.charges = x.charges
    for _ in range(max(args.warmup, 1)):
        Heff(x, out=y)
    ctx.synchronize()
    if args.describe:
        log("operator steps:\n" + Heff.describe())
    ctx.profile_begin()
    for _ in range(args.steps):
        Heff(x, out=y)
    prof = ctx.profile_end()
    t = prof["region_ms"] / 1e3
    g = prof["grouped"]
    per = g["flops"] / max(1, args.steps)
    line = {
        "metric": "H_eff TFLOP/s (charge blocks), two-site operator at the central bond",
        "value": g["flops"] / t / 1e12 if t > 0 else 0.0, "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": f"f64 ({args.precision} split contractions)", "data": "synthetic",
        "config": {"workload": f"J1-J2 {args.Ly}x{args.Lx} cylinder AC2 apply at bond {pos}, "
                               f"D={D}, U(1)", "terms": Heff.terms},
        "block_flops_per_matvec": per,
        "grouped_gemm": {"ms": g["ms"], "launches": g["launches"],
                         "tflops": g["flops"] / (g["ms"] / 1e3) / 1e12 if g["ms"] > 0 else 0.0},
        "gpu_launches": ctx.kernel_launches(),
    }
    print(json.dumps(line), flush=True)


def run_dmrg2_sweep(args):
    """Full DMRG2 sweeps (dmrg.jl:286-354: L-1 bond updates left to right, L-2 back) of the
    headline workload from its seeded random state, measured end to end: every local update
    (operator build, Galerkin matvec, adaptive Lanczos, blockwise truncated SVD) and every
    environment step.  Environments at D = 2048 are 2 GB each as dense embeddings: by default
    every one stays resident tile-packed (about a tenth of that) and the two in use are
    unpacked; with --env-storage checkpoint only every `checkpoint`-th one stays (dense) and
    the others are recomputed from the nearest, inside the measured sweep."""
    import mpsgb
    ctx = mpsgb.context(0)
    prec = args.precision
    ctx.set_precision(prec)
    ctx.set_svd_method(args.svd)
    ctx.set_gauge(args.eig, args.lanes)
    ctx.set_gemm_schedule(args.schedule, args.tile_n)
    backend = mpsgb.GB300Backend(prec, 0)
    H = mpsgb.j1j2_cylinder(args.Lx, args.Ly, dtype=np.float64, u1=True)
    n, D = len(H), args.D
    As, qb = mpsgb.u1.random_u1_tensors(n, D, args.seed, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=0,
                                       charges=(qb, mpsgb.operators.SPIN_HALF_CHARGES))
    del As
    K = max(1, args.checkpoint)
    if args.env_storage == "packed":
        # every environment resident, tile-packed but for the two in use
        envs = mpsgb.FiniteEnvironments(psi, H, packed=True)
    else:
        envs = mpsgb.FiniteEnvironments(psi, H, resident=False,
                                        keep_left=set(range(0, n + 1, K)),
                                        keep_right=set(range(0, n, K)))
    envs.precision = backend.code
    envs.rightenv(0, psi)
    ctx.synchronize()
    log("sweep workload: state and right environments ready")
    alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-10, backend=backend)
    with ClockSampler(0) as clocks:
        ctx.synchronize()
        t0 = time.perf_counter()
        psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, alg, envs=envs, maxsweeps=args.sweeps)
        ctx.synchronize()
        t = time.perf_counter() - t0
    per = [{"sweep": h["sweep"], "seconds": h["time"], "energy": h["energy"], "eps": h["eps"],
            "matvecs": h["matvecs"]} for h in hist]
    line = {
        "metric": "DMRG2 sweep seconds at D=2048 (J1-J2 6x24 cylinder, U(1))",
        "value": t / len(hist), "unit": "s/sweep", "n_gpus": 1, "steps": len(hist), "warmup": 0,
        "ms_per_step": 1e3 * t / len(hist), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": f"f64 ({prec} split contractions)", "data": "synthetic",
        "config": {"workload": f"J1-J2 Heisenberg {args.Ly}x{args.Lx} cylinder ({n} sites), full "
                               f"DMRG2 sweeps from the seeded random U(1) state (Sz = 0), "
                               f"D={D}, Float64", "env_storage": args.env_storage,
                   "checkpoint": K if args.env_storage == "checkpoint" else None,
                   "precision": prec},
        "sweeps": per, "clocks": clocks.summary(),
        "gpu_launches": ctx.kernel_launches(),
    }
    print(json.dumps(line), flush=True)


def run_vumps_sweep(args):
    """64 TFIM chains (J = 1, g uniformly in [0.1, 2.0], D drawn from {64, 128, 192, 256},
    ComplexF64), a fixed number of VUMPS iterations each, solved by `--workers` concurrent
    contexts; the same sweep solved one instance at a time is timed beside it."""
    import mpsgb
    from mpsgb import batched as B
    from oracle import models as M
    prec = args.precision
    alg = mpsgb.VUMPS(tol=1e-10, maxiter=args.vumps_iters, backend=mpsgb.GB300Backend(prec))
    ctxs = [mpsgb.Context(0) for _ in range(max(1, args.workers))]
    B.solve_vumps_batched(B.tfim_sweep(n=4, dims=(64,)), alg, contexts=ctxs[:4])  # warm-up
    log("vumps sweep warm-up done")
    res = {}
    for label, cs in (("concurrent", ctxs), ("sequential", ctxs[:1])):
        inst = B.tfim_sweep()
        for c in cs:
            c.synchronize()
        t0 = time.perf_counter()
        B.solve_vumps_batched(inst, alg, contexts=cs)
        t = time.perf_counter() - t0
        its = sum(i.iterations for i in inst)
        err = max(abs(i.energy - M.tfim_infinite_energy_density(i.label["g"])) for i in inst)
        res[label] = {"seconds": t, "iterations": its, "iter_per_s": its / t,
                      "max_energy_error_vs_exact": err}
        log(f"vumps sweep {label}: {t:.2f} s, {its} iterations")
    c = res["concurrent"]
    line = {
        "metric": "VUMPS iterations/s, 64-chain TFIM coupling sweep", "value": c["iter_per_s"],
        "unit": "VUMPS iterations/s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": 1e3 * c["seconds"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128" if prec == "fp64" else f"c128 ({prec} split contractions)",
        "data": "synthetic",
        "config": {"workload": "64 TFIM chains, J=1, g uniform in [0.1, 2.0], one-site VUMPS, "
                               "D drawn from {64,128,192,256} (seed 1238), ComplexF64",
                   "vumps_iterations_per_instance": args.vumps_iters, "workers": len(ctxs),
                   "precision": prec},
        "concurrent": c, "sequential": res["sequential"],
        "speedup_concurrent_vs_sequential": res["sequential"]["seconds"] / c["seconds"],
    }
    print(json.dumps(line), flush=True)


def run_vumps_xxz(args):
    """XXZ chain Jxy = 1, Jz = 1.5, hz = 0 (Neel phase) after a rotation by pi about x on
    every other site -- Jxy (SxSx - SySy) - Jz SzSz per bond, the same spectrum, one-site
    translation invariant -- one-site VUMPS, D = 256, ComplexF64 seeded random InfiniteMPS:
    the same iteration budget in plain FP64 and in split precision (tf32x3 unless
    --precision names another split mode); energies from FP64 environments of the final
    state, compared with the Bethe-ansatz energy density."""
    import mpsgb
    from mpsgb import _lib as L
    D = 256
    ctx = mpsgb.context(0)
    delta = 1.5
    H = mpsgb.xxz(1, 1.0, delta, 0.0, dtype=np.complex128, infinite=True, rotated=True)
    # Bethe ansatz for Delta = cosh(phi) > 1 (Yang and Yang 1966):
    # e = Delta/4 - sinh(phi) (1/2 + 2 sum_n 1/(exp(2 n phi) + 1))
    phi = np.arccosh(delta)
    n = np.arange(1, 2000)
    exact = delta / 4 - np.sinh(phi) * (0.5 + 2 * np.sum(1 / (np.exp(np.minimum(2 * n * phi, 700)) + 1)))
    rng = np.random.default_rng(args.seed)
    A = (rng.standard_normal((D, 2, D)) + 1j * rng.standard_normal((D, 2, D))).astype(np.complex128)
    split = args.precision if args.precision != "bf16x3" else "tf32x3"
    res = {}
    for prec in ("fp64", split):
        alg = mpsgb.VUMPS(tol=1e-10, maxiter=args.vumps_iters, backend=mpsgb.GB300Backend(prec))
        psi = mpsgb.InfiniteMPS.from_tensor(A, ctx)
        ctx.synchronize()
        t0 = time.perf_counter()
        psi, envs, eps, hist = mpsgb.find_groundstate_vumps(psi, H, alg)
        ctx.synchronize()
        t = time.perf_counter() - t0
        env64 = mpsgb.InfiniteEnvironments(psi, H, L.GB_PREC_FP64)
        env64.recalculate(psi, tol=1e-12)
        e = mpsgb.infinite.energy_density(psi, env64)
        phases = {}
        for h in hist:
            for k_, v_ in h["phase_s"].items():
                phases[k_] = phases.get(k_, 0.0) + v_ / len(hist)
        res[prec] = {"seconds": t, "iterations": len(hist), "s_per_iteration": t / len(hist),
                     "energy_density": e, "error_vs_exact": e - exact, "galerkin_eps": eps,
                     "phase_s_per_iteration": phases,
                     "matvecs_per_iteration": {
                         "ac": sum(h["matvecs"]["ac"] for h in hist) / len(hist),
                         "c": sum(h["matvecs"]["c"] for h in hist) / len(hist)}}
        log(f"vumps xxz {prec}: {t:.2f} s, {len(hist)} iterations, e = {e:.12f} "
            f"(exact {exact:.12f}), eps = {eps:.2e}")
    line = {
        "metric": "VUMPS s per iteration, XXZ (Jz = 1.5, sublattice-rotated) one-site cell, D = 256",
        "value": res[split]["s_per_iteration"], "unit": "s/iteration", "n_gpus": 1,
        "steps": args.vumps_iters, "warmup": 0, "ms_per_step": 1e3 * res[split]["s_per_iteration"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": f"c128 ({split} split contractions)", "data": "synthetic",
        "config": {"workload": "XXZ Jxy=1, Jz=1.5, hz=0 rotated by pi about x on odd sites, "
                               "one-site VUMPS, D=256, ComplexF64 "
                               f"random InfiniteMPS (seed {args.seed})",
                   "vumps_iterations": args.vumps_iters},
        "fp64": res["fp64"], "split": res[split],
        "split_speedup_per_iteration": res["fp64"]["s_per_iteration"] / res[split]["s_per_iteration"],
        "energy_difference": abs(res["fp64"]["energy_density"] - res[split]["energy_density"]),
    }
    print(json.dumps(line), flush=True)


def run_grassmann(args):
    """GradientGrassmann on a finite chain: TFIM at its critical point (g = 1), L = 64,
    D = 128, ComplexF64, seeded random state.  One step = one evaluation of the cost and
    gradient at a new point (grassmann.jl:150-169: environments of the new AL/AR, the energy,
    one AC projection per site, the Grassmann projection) plus the retraction that produced
    the point; after the timed steps a short CG run reports the gradient-norm decay.
    cpu_baseline: the oracle's fg at the same point on the host cores."""
    import mpsgb
    from mpsgb import grassmann as G
    from oracle import grassmann as OG
    from oracle import models as M
    from oracle import mps as P
    L_, D, gx = 64, 128, 1.0
    ctx = mpsgb.context(0)
    H = mpsgb.transverse_field_ising(L_, g=gx)
    As = P.random_initial_tensors(L_, 2, D, args.seed)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
    x = G.GrassmannPoint.from_state(psi)
    envs = mpsgb.FiniteEnvironments(x.psi, H, ctx)
    f, g = G.fg(x, H, envs)
    d = G.scale(G.precondition(x, g), -1.0)
    a = 1e-3
    n0 = ctx.kernel_launches()

    phase = {"retract": 0.0, "fg": 0.0, "precondition": 0.0}

    def step(k):
        t_ = time.perf_counter()
        xn, _ = G.retract(x, d, a * (1 + k))
        ctx.synchronize()
        phase["retract"] += time.perf_counter() - t_
        t_ = time.perf_counter()
        out = G.fg(xn, H, envs)
        ctx.synchronize()
        phase["fg"] += time.perf_counter() - t_
        t_ = time.perf_counter()
        G.precondition(xn, out[1])
        ctx.synchronize()
        phase["precondition"] += time.perf_counter() - t_
        return out

    for k in range(args.warmup):
        step(k)
    for key in phase:
        phase[key] = 0.0
    ctx.synchronize()
    n0 = ctx.kernel_launches()
    t0 = time.perf_counter()
    for k in range(args.steps):
        fk, _ = step(args.warmup + k)
    ctx.synchronize()
    t = (time.perf_counter() - t0) / args.steps
    launches = ctx.kernel_launches() - n0
    log(f"grassmann: {1e3 * t:.1f} ms per retract + fg + precondition, {launches} launches")
    # a short optimisation from the same state
    t1 = time.perf_counter()
    _, _, ng, hist = mpsgb.find_groundstate(mpsgb.FiniteMPS.from_tensors(As, ctx), H,
                                            mpsgb.GradientGrassmann(tol=1e-8, maxiter=20))
    t_opt = time.perf_counter() - t1
    cpu = None
    if not args.no_cpu_baseline:
        oH = M.finite_mpo_hamiltonian(L_, 2, M.tfim_terms(L_, g=gx))
        AL = [a_.numpy() for a_ in x.AL]
        Cend = x.psi.C[L_].numpy()
        od = [t_.Z.numpy() for t_ in d]
        of, og = OG.fg(AL, Cend, oH)
        t2 = time.perf_counter()
        ALn, Cn, _ = OG.retract(AL, Cend, od, a)
        of2, og2 = OG.fg(ALn, Cn, oH)
        OG.precondition(ALn, Cn, og2)
        tc = time.perf_counter() - t2
        cpu = {"value": tc, "unit": "s/fg", "cores": os.cpu_count(), "kind": "port",
               "sample": "one oracle line-search point (retract of the 64 sites, fg: "
                         "environments, energy, 64 AC projections; precondition) from the "
                         "device's first point along the same direction; numpy/BLAS",
               "energy_difference": abs(of - f)}
    line = {
        "metric": ("GradientGrassmann s per line-search point (retract + fg + precondition), "
                   "TFIM g=1, L=64, D=128"),
        "value": t, "unit": "s/fg", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128 (fp64)", "data": "synthetic",
        "config": {"workload": "finite TFIM g=1 L=64, D=128, ComplexF64, seeded random MPS; "
                               "step = retraction + fg + precondition", "l2": "working set < L2"},
        "gpu_launches": launches,
        "phase_s_per_step": {k_: v_ / args.steps for k_, v_ in phase.items()},
        "cg_20_iterations": {"seconds": t_opt, "fg_evaluations": hist["numfg"],
                             "normgrad_first_last": [hist["normgrad"][0], hist["normgrad"][-1]],
                             "energy": hist["energy"]},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "vumps-sweep":
        run_vumps_sweep(args)
    elif args.workload == "matvec":
        run_matvec(args)
    elif args.workload == "dmrg2-sweep":
        run_dmrg2_sweep(args)
    elif args.workload == "vumps-xxz":
        run_vumps_xxz(args)
    elif args.workload == "grassmann":
        run_grassmann(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
