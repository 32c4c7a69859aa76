"""Benchmark: BLS12-381 G1 multiexp throughput (Mpts/s) at n = 2^20.

Workload: the 2^20-point KZG commitment MSM of the "Fr NTT + coset LDE"
configuration -- uniform Fr scalars (Montgomery form), bases [r_i] G with
uniform r_i, seeded synthetic data.  One step = one 2^20 MSM through the
resident-bases context (the reference's `Bls12_381G1MsmContext` path that
KZG commitments use).

  value : Mpts/s with scalars already resident in HBM (device-vector entry
          point, result copied back to the host each step)
  e2e   : Mpts/s through the host-buffer context entry point; every step
          copies its 32 MiB of scalars host->device and the 144-byte result back

Also reported: the roofline of the dominant kernel (bucket accumulation)
against the measured 32x32->64 multiply-add peak, the whole-MSM roofline,
the plain (non-resident) MSM, NTT/LDE timings of the same configuration, and
the oracle's CPU multiexp on this host as the CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb|reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "midnight-ledger-cuda_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

R_MOD = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
R_LIMBS = np.array([(R_MOD >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(4)], dtype=np.uint64)
METRIC = "G1 MSM Mpts/s at 2^20"
FP_MULS_PER_MADD = 10    # XYZZ mixed addition: 8M + 2S
FP_MULS_PER_ADD = 14     # XYZZ addition: 12M + 2S
MADDS_PER_FP_MUL = 300   # 2 * 12^2 + 12 32x32->64 multiply-adds per Fp product
ACC_DRAM_BYTES_PER_ENTRY = 801.33e6 / ((1 << 18) * 16)  # ncu, n = 2^18 launch (c = 16: 16 windows)


def fr_uniform(n, rng):
    """Uniform Fr values by rejection (Fq::random style), as Montgomery limbs."""
    out = np.empty((n, 4), dtype=np.uint64)
    filled = 0
    while filled < n:
        k = int((n - filled) * 1.3) + 16
        c = rng.integers(0, 2**64, size=(k, 4), dtype=np.uint64)
        c[:, 3] &= np.uint64(0x7FFFFFFFFFFFFFFF)
        lt = np.zeros(k, dtype=bool)
        eq = np.ones(k, dtype=bool)
        for i in (3, 2, 1, 0):
            lt |= eq & (c[:, i] < R_LIMBS[i])
            eq &= c[:, i] == R_LIMBS[i]
        c = c[lt]
        t = min(len(c), n - filled)
        out[filled:filled + t] = c[:t]
        filled += t
    return out


def windows(c):
    return 254 // c + 1


def f_msm(n):
    """Algorithmic Fp products of an n-point MSM with uniform scalars:
    min over c in [8, 20] of 10 n W(c) + 14 W(c) 2^c, W(c) = floor(254/c)+1.
    Returns (total, mixed-addition term, c)."""
    best = None
    for c in range(8, 21):
        w = windows(c)
        madd = FP_MULS_PER_MADD * n * w
        tot = madd + FP_MULS_PER_ADD * w * (1 << c)
        if best is None or tot < best[0]:
            best = (tot, madd, c)
    return best


_MAX_MHZ = []


def issue_ceiling_tmadd():
    """The multiply-add issue ceiling in T products/s: the IMAD pipe takes 64
    lanes per clock per SM and a 32x32->64 product is two instructions
    (mad.lo + madc.hi), so 32 products per clock per SM x SMs x the maximum
    SM clock (nvidia-smi clocks.max.sm)."""
    import torch
    if not _MAX_MHZ:
        mhz = 2070.0
        try:
            r = subprocess.run(["nvidia-smi", "-i", str(torch.cuda.current_device()), "--query-gpu=clocks.max.sm",
                                "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=10)
            mhz = float(r.stdout.strip().splitlines()[0])
        except (OSError, ValueError, IndexError, subprocess.TimeoutExpired):
            pass
        _MAX_MHZ.append(mhz)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return 32 * sms * _MAX_MHZ[0] * 1e6 / 1e12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms.  The
    sampler is running before the timed region starts (its first row has
    arrived), each row carries its arrival time, and the summary keeps the
    rows that arrived inside the region set by window()."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index, interval_ms=20):
        self.index = index
        self.interval_ms = interval_ms
        self.rows = []
        self.proc = None
        self.span = None
        self.first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            self.first.wait(timeout=5.0)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append((time.perf_counter(), parts))
                self.first.set()

    def window(self, t0, t1):
        """the timed region, in time.perf_counter() seconds"""
        self.span = (t0, t1)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(2 * self.interval_ms / 1e3)  # the row covering the region's end
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = [r for t, r in self.rows if self.span is None or self.span[0] <= t <= self.span[1] +
                self.interval_ms / 1e3]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "interval_ms": self.interval_ms}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("GB_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_bases(n, seed):
    """Bases [r_i]G for the CPU baseline (generated once, outside any timing)."""
    from oracle import oracle as orc
    return orc.g1_generator_mul_batch(fr_uniform(n, np.random.default_rng(seed)))


def cpu_baseline_msm(n, seed, b=None):
    """The oracle's multithreaded CPU Pippenger (a C restatement of the
    reference's msm_best / blst semantics) on this host's cores; the bases
    are made here unless given."""
    from oracle import oracle as orc
    rng = np.random.default_rng(seed)
    s = fr_uniform(n, rng)
    if b is None:
        b = orc.g1_generator_mul_batch(fr_uniform(n, rng))
    threads = os.cpu_count() or 1
    orc.g1_msm(b[:1024], s[:1024], threads=threads)
    t0 = time.perf_counter()
    orc.g1_msm(b, s, threads=threads)
    dt = time.perf_counter() - t0
    return n / dt / 1e6, threads, dt


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU multiexp semantics on the host
    cores.  The reference's own CPU path (Rust: blst + rayon) cannot be built
    in this image, so the oracle's C restatement stands in for it."""
    if rank != 0:
        return
    n = args.n_ref
    bases = cpu_bases(n, 999)
    vals, dts, threads = [], [], 1
    for i in range(args.warmup + args.steps):
        v, threads, dt = cpu_baseline_msm(n, 1000 + i, bases)
        if i >= args.warmup:
            vals.append(v)
            dts.append(dt)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(dts) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 limbs (exact Fp/Fr)",
        "data": "synthetic (seeded uniform Fr scalars, bases [r_i]G)",
        "config": {"workload": "G1 MSM n=2^%d, uniform Fr scalars, bases [r_i]G: KZG commitment of the "
                               "16x2^20 NTT + coset LDE configuration" % args.log_n,
                   "n": args.n, "sample_n": n, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "Mpts/s", "cores": threads, "kind": "port",
                         "sample": "one n=2^%d MSM of the same scalar/base distribution per step (the 2^%d "
                                   "workload's size; fresh scalars each step, bases made once; oracle C "
                                   "Pippenger on all host threads); the reference's Rust CPU path is not "
                                   "buildable here" % (n.bit_length() - 1, args.log_n)},
        "e2e": {"value": value, "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb", choices=["gb", "reference"])
    ap.add_argument("--log-n", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--case", default="msm", choices=["msm", "ntt", "ntt-queue", "proof"],
                    help="msm: the benchmark line; ntt / ntt-queue: only the resident NTT batch of --count "
                         "transforms of 2^--log-n, or the 64-transform ragged batch in one launch; proof: "
                         "--steps k=16 proofs after the key generation and --warmup proofs, with a "
                         "peak_row_kernel launch just before the last proof as a marker (small cases for "
                         "profilers; one JSON line of timings)")
    ap.add_argument("--count", type=int, default=16)
    ap.add_argument("--circuit", type=int, default=-1,
                    help="--case proof: -1 = the k = 16 configuration, 0..5 = one of the serving mix's circuits")
    args = ap.parse_args()
    args.n = 1 << args.log_n
    args.n_ref = args.n  # the CPU baseline runs the whole 2^20 MSM (about 2 s on 16 Grace cores)
    args.warmup = max(args.warmup, 3) if args.impl == "gb" else args.warmup
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.case == "proof":
        run_proof_case(args)
        return
    if args.case != "msm":
        run_ntt_case(args)
        return

    import torch
    import gb_prover as gb

    torch.cuda.set_device(local)
    gb.lib()
    n = args.n
    rng = np.random.default_rng(20 + rank)
    nsets = 8  # 8 x 32 MiB scalar sets rotate through the steps (256 MiB > L2)
    scalars = fr_uniform(n * nsets, rng)
    bases = gb.g1_generator_mul(fr_uniform(n, rng))
    ctx = gb.Bls12_381G1MsmContext(bases)
    dv = gb.Bls12_381FrDeviceVec.upload(scalars)
    stream = torch.cuda.ExternalStream(gb.lane_stream())

    def step(i):
        return ctx.device_batch(dv, (i % nsets) * n, n, 1)

    for i in range(args.warmup):
        step(i)
    probe_forms = [gb.imad_probe(f) for f in range(4)]
    peak = max(probe_forms)

    # ---- timed region: device-resident scalars
    gb.profile_reset()
    gb.profile_enable(True)
    launches0 = gb.launch_counter()
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t0 = time.perf_counter()
        for i in range(args.steps):
            step(i)
        e1.record(stream)
        e1.synchronize()
        wall = time.perf_counter() - t0
        clk.window(t0, t0 + wall)
    torch.cuda.synchronize()
    barrier(world)
    launches = gb.launch_counter() - launches0
    gb.profile_enable(False)
    dev_ms = e0.elapsed_time(e1)
    dev_ms = max_over_ranks(dev_ms, world)
    acc_ms, acc_n = gb.profile_read(gb.PROFILE_MSM_ACCUMULATE)
    msm_ms, msm_n = gb.profile_read(gb.PROFILE_MSM_TOTAL)
    value = world * n * args.steps / (dev_ms * 1e-3) / 1e6

    # ---- e2e: host scalars in pinned memory through the host-buffer entry
    pinned = torch.empty((nsets, n, 4), dtype=torch.int64, pin_memory=True)
    pinned.numpy().view(np.uint64)[:] = scalars.reshape(nsets, n, 4)
    host = pinned.numpy().view(np.uint64)
    for i in range(2):
        ctx.batch(host[i])
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        ctx.batch(host[i % nsets])
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = world * n * args.steps / e2e_s / 1e6

    # ---- roofline
    total_fp, madd_fp, c_star = f_msm(n)
    acc_avg_s = acc_ms / max(acc_n, 1) * 1e-3
    msm_avg_s = msm_ms / max(msm_n, 1) * 1e-3
    acc_ops = madd_fp * MADDS_PER_FP_MUL
    achieved = acc_ops / acc_avg_s / 1e12 if acc_avg_s else None
    roofline = {
        "bound": "imad", "unit": "Tmadd/s",
        "kernel": "msm_accumulate_kernel",
        "achieved": achieved, "peak": peak / 1e12, "frac": achieved / (peak / 1e12) if achieved else None,
        "peak_source": "measured live: gb_imad_probe, the fastest of mad.wide.u32 chains and carry-chained 12-limb "
                       "rows (1, 2, 4 accumulator sets per thread) with operands that change every iteration, all SMs; "
                       "unit = one 32x32->64 product",
        "peak_forms": {"wide": probe_forms[0] / 1e12, "rows1": probe_forms[1] / 1e12,
                       "rows2": probe_forms[2] / 1e12, "rows4": probe_forms[3] / 1e12},
        "algorithmic_per_launch": "10 Fp-mul x n x W(c*) mixed additions, c*=%d, W=%d, 300 madd per Fp-mul"
                                  % (c_star, windows(c_star)),
        "avg_launch_ms": acc_avg_s * 1e3, "launches": acc_n,
        # DRAM bytes of one accumulate launch: the ncu capture of the n=2^18
        # launch (dram__bytes_read.sum + dram__bytes_write.sum = 801.33 MB over
        # 2^18 x 16 digit entries) scaled by this launch's n x W entries
        "traffic": ACC_DRAM_BYTES_PER_ENTRY * n * windows(c_star),
        "traffic_source": "ncu capture at n=2^18, scaled per digit entry",
    }
    roofline_msm = {
        "bound": "imad", "unit": "Tmadd/s", "F_msm_fp_mul": total_fp,
        "achieved": total_fp * MADDS_PER_FP_MUL / msm_avg_s / 1e12 if msm_avg_s else None,
        "peak": peak / 1e12, "avg_msm_ms": msm_avg_s * 1e3,
    }
    roofline_msm["frac"] = roofline_msm["achieved"] / roofline_msm["peak"] if roofline_msm["achieved"] else None
    ceiling = issue_ceiling_tmadd()
    roofline["issue_ceiling"] = ceiling
    roofline["frac_issue_ceiling"] = achieved / ceiling if achieved else None
    roofline["issue_ceiling_source"] = ("32 products per clock per SM (64 IMAD lanes, 2 instructions per "
                                        "32x32->64 product) x SMs x max SM clock")
    roofline_msm["frac_issue_ceiling"] = roofline_msm["achieved"] / ceiling if roofline_msm["achieved"] else None

    extra = {}
    if not args.no_extras:
        extra = extras(gb, torch, n, rng, bases, args, peak)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, threads, dt = cpu_baseline_msm(args.n_ref, 77)
        cpu = {"value": v, "unit": "Mpts/s", "cores": threads, "kind": "port",
               "sample": "one n=2^%d MSM (same scalar/base distribution), oracle C Pippenger on all host "
                         "threads (%.1f s)" % (args.n_ref.bit_length() - 1, dt)}
        if not args.no_extras:
            cpu["proof_k16_s"] = cpu_baseline_proof()
            cpu["ntt_2p20_ms"] = cpu_baseline_ntt(20)

    del ctx, dv
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mpts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 limbs (exact Fp/Fr Montgomery)",
            "data": "synthetic (seeded uniform Fr scalars, bases [r_i]G)",
            "config": {"workload": "G1 MSM n=2^%d, uniform Fr scalars, bases [r_i]G: KZG commitment of the "
                                   "16x2^20 NTT + coset LDE configuration, resident-bases context"
                                   % args.log_n,
                       "n": n, "l2": "inputs larger than L2: 2^20 x 16-window base table (1.5 GiB) and 8 "
                                     "rotating 32 MiB scalar sets", "parallelism": "replicas" if world > 1 else "1gpu",
                       "table_bytes": n * windows(c_star) * 96,
                       "table": "the context keeps 2^(16 j) P_i for the 16 windows j (fixed-base precomputation "
                                "over the resident SRS; every digit still costs one mixed addition); "
                                "extra.msm_2p20_resident_no_table_ms is the same MSM without it"},
            "e2e": {"value": e2e, "unit": "Mpts/s", "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": 144},
            "gpu_launches": launches,
            "wall_s": wall,
            "roofline": roofline,
            "roofline_msm": roofline_msm,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "extra": extra,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_proof_case(args):
    """--case proof: the k = 16 synthetic proof (or, with --circuit i, the
    serving mix's circuit i), one at a time (wall time)."""
    import torch
    import gb_prover as gb
    from gb_prover import plonk
    from gb_prover.kzg import CircuitTranscript, ParamsKZG
    from gb_prover.rng import ChaCha20Rng, ints_to_mont
    torch.cuda.set_device(0)
    gb.lib()
    if args.circuit < 0:
        k = 16
        c = plonk.SyntheticCircuit(16, advice=3, degree=3, lookups=1, copies=1 << 14, table_log=12,
                                   label="full synthetic PLONK/KZG proof, k=16")
    else:
        k, m, d, L, _ = SERVE_CIRCUITS[args.circuit]
        c = plonk.SyntheticCircuit(k, advice=m, degree=d, lookups=L, copies=1 << (k - 2),
                                   table_log=min(12, k - 3), label="serve circuit %d" % args.circuit)
    fixed, advice, copies = c.synthesize()
    params = ParamsKZG.unsafe_setup(k, plonk.fr_mont(0x5EED0F7A0))
    be = plonk.GpuBackend(params)
    pk = plonk.keygen(params, c, be, fixed, copies)
    adv = ints_to_mont([v for col in advice for v in col])
    for i in range(args.warmup):
        plonk.create_proof(params, pk, adv, be, CircuitTranscript(), ChaCha20Rng.from_label("warm%d" % i))
    ms = []
    for i in range(args.steps):
        if i == args.steps - 1:
            gb.imad_probe(1)
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        plonk.create_proof(params, pk, adv, be, CircuitTranscript(), ChaCha20Rng.from_label("p%d" % i))
        ms.append((time.perf_counter() - t0) * 1e3)
    print(json.dumps({"case": "proof", "k": k, "circuit": args.circuit, "ms": ms, "best_ms": min(ms)}))


def run_ntt_case(args):
    """--case ntt | ntt-queue: resident forward NTTs only, timed with CUDA
    events on the library's lane stream (W untimed, K timed calls)."""
    import torch
    import gb_prover as gb
    torch.cuda.set_device(0)
    gb.lib()
    rng = np.random.default_rng(7)
    one = np.array([0x00000001FFFFFFFE, 0x5884B7FA00034802, 0x998C4FEFECBC4FF5, 0x1824B159ACC5056F], np.uint64)
    if args.case == "ntt":
        logs = [args.log_n] * args.count
    else:
        logs = sorted((max(1, (int(round(2 ** u)) - 1).bit_length()) for u in rng.uniform(10, 18, size=64)),
                      reverse=True)
    offs = np.concatenate([[0], np.cumsum([1 << lg for lg in logs])[:-1]]).astype(np.uint64)
    dv = gb.Bls12_381FrDeviceVec.upload(fr_uniform(int(sum(1 << lg for lg in logs)), rng))

    def call():
        if args.case == "ntt":
            dv.ntt_zeta_batch(args.log_n, args.count, False, one, one, one)
        else:
            dv.ntt_ragged(offs, logs, False, one, one, one)

    stream = torch.cuda.ExternalStream(gb.lane_stream())
    for _ in range(args.warmup):
        call()
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    fr_mul = sum((1 << (lg - 1)) * lg for lg in logs)
    print(json.dumps({"case": args.case, "transforms": len(logs), "elements": int(sum(1 << lg for lg in logs)),
                      "ms": ms, "best_ms": min(ms), "tmadd_per_s": fr_mul * 136 / min(ms) / 1e9}))


def mixed_scalars(n, rng):
    """70% uniform Fr, 20% uniform below 2^64, 10% zero."""
    s = fr_uniform(n, rng)
    u = rng.random(n)
    small = (u >= 0.7) & (u < 0.9)
    k = int(small.sum())
    s[small] = 0
    # a uniform value below 2^64 in Montgomery form: v * R mod r, computed exactly
    vals = rng.integers(0, 2**63, size=k, dtype=np.int64).astype(object) * 2 + rng.integers(0, 2, size=k)
    R = pow(2, 256, R_MOD)
    mont = [(int(v) * R) % R_MOD for v in vals]
    s[small] = np.array([[(m >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(4)] for m in mont],
                        dtype=np.uint64).reshape(-1, 4)
    s[u >= 0.9] = 0
    return s


CONFIG4_SEED = 4004


def config4_inputs(seed=CONFIG4_SEED):
    """The batched MSM/NTT configuration's inputs: 64 MSM sizes round(2^U),
    U ~ U[10, 18]; their scalars (70% uniform Fr, 20% uniform below 2^64,
    10% zero); the scalars of the 2^18 base set (bases [r_i] G); and the
    NTT sizes (the next power of two of each MSM size).  Seeded, so the
    parity test checks exactly the batch this benchmark times."""
    rng = np.random.default_rng(seed)
    sizes = [int(round(2 ** u)) for u in rng.uniform(10, 18, size=64)]
    base_scalars = fr_uniform(1 << 18, rng)
    scal = [mixed_scalars(n, rng) for n in sizes]
    logs = [max(1, (n - 1).bit_length()) for n in sizes]
    return sizes, scal, base_scalars, logs


def batched_config(gb, torch, rng):
    """64 MSMs with sizes round(2^U), U ~ U[10, 18], the 70/20/10 scalar mix,
    against a resident 2^18 SRS-like base set: one batched call versus one
    call per MSM; and 64 NTTs of the matching power-of-two sizes, batched per
    size versus one call per NTT."""
    sizes, scal, base_scalars, logs = config4_inputs()
    bases = gb.g1_generator_mul(base_scalars)
    ctx = gb.Bls12_381G1MsmContext(bases)
    flat = np.concatenate(scal)
    dv = gb.Bls12_381FrDeviceVec.upload(flat)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int)
    slices = [(int(o), 0, n) for o, n in zip(offs, sizes)]
    stream = torch.cuda.ExternalStream(gb.lane_stream())

    def timed(fn):
        return median_ms(torch, stream, fn)

    batched = timed(lambda: ctx.device_ragged(dv, slices))
    single = timed(lambda: [ctx.device_ragged(dv, [sl]) for sl in slices])
    out = {"msm64_total_points": int(sum(sizes)), "msm64_batched_ms": batched, "msm64_one_at_a_time_ms": single,
           "msm64_batched_mpts_s": sum(sizes) / batched / 1e3}
    # NTTs: next power of two of each size
    polys = {lg: fr_uniform((1 << lg) * logs.count(lg), rng) for lg in set(logs)}
    one = np.array([0x00000001FFFFFFFE, 0x5884B7FA00034802, 0x998C4FEFECBC4FF5, 0x1824B159ACC5056F], np.uint64)
    vecs = {lg: gb.Bls12_381FrDeviceVec.upload(v) for lg, v in polys.items()}
    singles = {lg: [gb.Bls12_381FrDeviceVec.upload(polys[lg][i << lg:(i + 1) << lg]) for i in range(logs.count(lg))]
               for lg in set(logs)}
    out["ntt64_batched_ms"] = timed(lambda: [vecs[lg].ntt_zeta_batch(lg, logs.count(lg), False, one, one, one)
                                             for lg in vecs])
    out["ntt64_one_at_a_time_ms"] = timed(lambda: [v.ntt_zeta(lg, False, one, one, one)
                                                   for lg in singles for v in singles[lg]])
    # all 64 NTTs, of every size, in one persistent launch fed by the device
    # work queue (one vector holding the 64 polynomials back to back)
    order = sorted(range(64), key=lambda j: -logs[j])
    q_logs = [logs[j] for j in order]
    q_offs = np.concatenate([[0], np.cumsum([1 << lg for lg in q_logs])[:-1]]).astype(np.uint64)
    qv = gb.Bls12_381FrDeviceVec.upload(fr_uniform(int(sum(1 << lg for lg in q_logs)), rng))
    out["ntt64_queue_ms"] = timed(lambda: qv.ntt_ragged(q_offs, q_logs, False, one, one, one))
    out["ntt64_queue_launches"] = 1
    del qv
    # the same two batches with the autotuner choosing the window and the NTT
    # pass variant (the first call of each key tunes; then timed as above)
    gb.autotune_reset()
    gb.autotune_set(True)
    try:
        out["msm64_autotuned_ms"] = timed(lambda: ctx.device_ragged(dv, slices))
        out["ntt64_autotuned_ms"] = timed(lambda: [vecs[lg].ntt_zeta_batch(lg, logs.count(lg), False, one, one, one)
                                                   for lg in vecs])
        out["autotuned"] = gb.autotune_report()
    finally:
        gb.autotune_set(False)
    del ctx, dv
    return out


def proof_config(gb, steps=10):
    """The full synthetic PLONK/KZG proof at k = 16 (3 advice columns,
    standard gate, 2^14 copy constraints, one 2-column lookup into a 2^12-row
    table, SRS of 2^16 points from a seeded tau): proofs one at a time
    through the GPU prover, the witness already in Montgomery form on the
    host, each proof ending with its bytes on the host."""
    from gb_prover import plonk
    from gb_prover.kzg import CircuitTranscript, ParamsKZG
    from gb_prover.rng import ChaCha20Rng, ints_to_mont
    c = plonk.SyntheticCircuit(16, advice=3, degree=3, lookups=1, copies=1 << 14, table_log=12,
                               label="full synthetic PLONK/KZG proof, k=16")
    fixed, advice, copies = c.synthesize()
    params = ParamsKZG.unsafe_setup(16, plonk.fr_mont(0x5EED0F7A0))
    be = plonk.GpuBackend(params)
    t0 = time.perf_counter()
    pk = plonk.keygen(params, c, be, fixed, copies)
    keygen_s = time.perf_counter() - t0
    adv = ints_to_mont([v for col in advice for v in col])
    for i in range(2):
        plonk.create_proof(params, pk, adv, be, CircuitTranscript(), ChaCha20Rng.from_label("warm%d" % i))
    lat = []
    for i in range(steps):
        t0 = time.perf_counter()
        proof = plonk.create_proof(params, pk, adv, be, CircuitTranscript(), ChaCha20Rng.from_label("p%d" % i))
        lat.append(time.perf_counter() - t0)
    lat.sort()
    out = {"proof_k16_proofs_per_s": steps / sum(lat), "proof_k16_p50_ms": lat[len(lat) // 2] * 1e3,
           "proof_k16_p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))] * 1e3,
           "proof_k16_bytes": len(proof), "proof_k16_keygen_s": keygen_s, "proof_k16_count": steps}
    # saturated throughput: 32 requests queued at once, one lane against several
    from gb_prover import serve
    for slots, lock in ((1, 1), (4, 1), (8, 1), (4, 4)):
        srv = serve.ProofServer({0: (params, pk)}, slots=slots, lockstep=lock)
        for i in range(slots * lock):
            srv.submit(0, adv, "warm%d" % i)
        srv.drain()
        t0 = time.perf_counter()
        reqs = [srv.submit(0, adv, "s%d" % i) for i in range(32)]
        for r in reqs:
            r.future.result()
        key = "%dlane" % slots + ("_lockstep%d" % lock if lock > 1 else "")
        out["proof_k16_saturated_%s_proofs_per_s" % key] = 32 / (time.perf_counter() - t0)
        srv.close()
    return out


SERVE_CIRCUITS = [  # (k, advice, gate degree, lookups, share of requests)
    (12, 3, 3, 0, 0.40), (13, 4, 4, 1, 0.25), (14, 8, 5, 2, 0.15),
    (15, 5, 3, 1, 0.10), (16, 3, 3, 1, 0.05), (18, 4, 4, 0, 0.05)]


def serve_config(gb, requests=160, slots=4, hbm_budget=8 << 30, loads=(0.85, 1.5)):
    """Proof serving: a Poisson stream of proof requests over 6 synthetic
    circuits (k = 12..18, 3-8 advice columns, gate degree 3-5, 0-2 lookups,
    request shares 40/25/15/10/5/5 %), the 2^18-point SRS (downsized per k)
    and every proving key resident.  The HBM budget covers everything: the
    resident SRS tables and keys are counted first and the proofs in flight
    share the rest.  The arrival rate loads the sequential prover to each of
    `loads` of its capacity (below and above it); each stream runs through
    the one-at-a-time prover (1 slot) and the continuous-batching server
    (`slots` lanes), without and with the proofs' commitments fused into
    shared MSM batches (CommitBatcher), and with lockstep groups of up to 4
    waiting requests of one circuit per lane (plonk.create_proofs).  The saturated throughput of the mix
    (every request queued at once) is measured the same three ways."""
    from gb_prover import plonk, serve
    from gb_prover.kzg import CircuitTranscript, ParamsKZG
    from gb_prover.rng import ChaCha20Rng, ints_to_mont
    t0 = time.perf_counter()
    srs = ParamsKZG.unsafe_setup(18, plonk.fr_mont(0x5EED0F7A0))
    entries, wits, shares, per_k = {}, {}, [], {18: srs}
    for cid, (k, m, d, L, share) in enumerate(SERVE_CIRCUITS):
        c = plonk.SyntheticCircuit(k, advice=m, degree=d, lookups=L, copies=1 << (k - 2),
                                   table_log=min(12, k - 3), label="serve circuit %d" % cid)
        fixed, advice, copies = c.synthesize()
        params = per_k.setdefault(k, srs.downsize(k))
        entries[cid] = (params, plonk.keygen(params, c, plonk.GpuBackend(params), fixed, copies))
        wits[cid] = ints_to_mont([v for col in advice for v in col])
        shares.append(share)
    for params in per_k.values():  # the contexts the server will hold
        params.context(True)
        params.context(False)
    setup_s = time.perf_counter() - t0
    resident = sum(p.device_bytes() for p in per_k.values()) + sum(pk.device_bytes() for _, pk in entries.values())
    proof_budget = hbm_budget - resident
    # sequential service time per circuit (after a warm-up proof each)
    service = []
    for cid, (params, pk) in entries.items():
        be = plonk.GpuBackend(params)
        plonk.create_proof(params, pk, wits[cid], be, CircuitTranscript(), ChaCha20Rng.from_label("warm"))
        t1 = time.perf_counter()
        for i in range(3):
            plonk.create_proof(params, pk, wits[cid], be, CircuitTranscript(), ChaCha20Rng.from_label("w%d" % i))
        service.append((time.perf_counter() - t1) / 3)
    mean_s = sum(sh * t for sh, t in zip(shares, service))
    rng = np.random.default_rng(2024)
    cids = rng.choice(len(shares), size=requests, p=np.array(shares) / sum(shares))
    reqs = [(int(c), wits[int(c)], "request-%d" % i) for i, c in enumerate(cids)]
    out = {"serve_setup_s": setup_s, "serve_requests": requests, "serve_service_ms": [t * 1e3 for t in service],
           "serve_sequential_capacity_per_s": 1 / mean_s, "serve_slots": slots,
           "serve_hbm_budget_gb": hbm_budget / 2 ** 30, "serve_resident_gb": resident / 2 ** 30,
           "serve_proof_budget_gb": proof_budget / 2 ** 30}
    proofs = {}
    for load in loads:
        rate = load / mean_s
        arrivals = serve.poisson_arrivals(np.random.default_rng(2025), rate, requests)
        tag = "load%03d" % int(round(load * 100))
        out["serve_%s_rate_per_s" % tag] = rate
        for name, nslots, fuse, lock in (("sequential", 1, False, 1), ("batched", slots, False, 1),
                                         ("fused", slots, True, 1), ("lockstep", slots, False, 4)):
            srv = serve.ProofServer(entries, slots=nslots, hbm_budget=proof_budget, fuse_commits=fuse, lockstep=lock)
            done, ts = serve.run_stream(srv, reqs, arrivals)
            srv.close()
            summ = serve.latency_summary(done, ts)
            for key in ("proofs_per_s", "p50_ms", "p99_ms", "mean_ms"):
                out["serve_%s_%s_%s" % (tag, name, key)] = summ[key]
            if fuse:
                out["serve_%s_fused_commit_batches" % tag] = srv.batcher.batches
                out["serve_%s_fused_commit_requests" % tag] = srv.batcher.fused_requests
            proofs[(tag, name)] = [r.future.result() for r in done]
    out["serve_batched_equals_sequential"] = all(proofs[(t, m)] == proofs[(t, "sequential")]
                                                 for t, m in proofs if m != "sequential")
    # saturated: the whole stream queued at once
    for name, nslots, fuse, lock in (("1lane", 1, False, 1), ("%dlane" % slots, slots, False, 1),
                                     ("8lane", 8, False, 1), ("%dlane_fused" % slots, slots, True, 1),
                                     ("%dlane_lockstep4" % slots, slots, False, 4), ("8lane_lockstep4", 8, False, 4)):
        srv = serve.ProofServer(entries, slots=nslots, hbm_budget=proof_budget, fuse_commits=fuse, lockstep=lock)
        done, ts = serve.run_stream(srv, reqs, [0.0] * requests)
        srv.close()
        out["serve_saturated_%s_proofs_per_s" % name] = serve.latency_summary(done, ts)["proofs_per_s"]
    return out


def cpu_baseline_ntt(log_n):
    """One forward Fr NTT of 2^log_n uniform values, the oracle's radix-2
    transform (the reference's best_fft semantics) on all host threads."""
    from oracle import oracle as orc
    v = fr_uniform(1 << log_n, np.random.default_rng(78))
    threads = os.cpu_count() or 1
    orc.fr_ntt(v[:1024], 10, False, threads=threads)
    t0 = time.perf_counter()
    orc.fr_ntt(v, log_n, False, threads=threads)
    return (time.perf_counter() - t0) * 1e3


def cpu_baseline_proof():
    """One k = 16 proof of the same circuit through the prover driver on the
    oracle's C restatements (all host threads)."""
    from gb_prover import plonk
    from gb_prover.kzg import CircuitTranscript
    from gb_prover.rng import ChaCha20Rng
    from oracle import plonk_cpu
    c = plonk.SyntheticCircuit(16, advice=3, degree=3, lookups=1, copies=1 << 14, table_log=12,
                               label="full synthetic PLONK/KZG proof, k=16")
    fixed, advice, copies = c.synthesize()
    params = plonk_cpu.setup_params(16, 0x5EED0F7A0)
    be = plonk_cpu.OracleBackend(params)
    pk = plonk.keygen(params, c, be, fixed, copies)
    t0 = time.perf_counter()
    plonk.create_proof(params, pk, advice, be, CircuitTranscript(), ChaCha20Rng.from_label("cpu"))
    return time.perf_counter() - t0


def median_ms(torch, stream, fn, reps=5):
    """median of `reps` CUDA-event timings of fn() on the library's lane
    stream (after one untimed call)"""
    fn()
    ms = []
    for _ in range(reps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return statistics.median(ms)


def median_wall_ms(torch, fn, reps=5):
    """median wall time of fn() (host buffers in and out), after one untimed call"""
    fn()
    ms = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        ms.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(ms)


def extras(gb, torch, n, rng, bases, args, peak):
    """Secondary numbers of the same configuration (not the headline); each
    figure is the median of 5 timed calls after an untimed one."""
    out = {}
    stream = torch.cuda.ExternalStream(gb.lane_stream())
    lib = gb.lib()
    # plain MSM: bases and scalars from host, nothing resident
    s = fr_uniform(n, rng)
    out["plain_msm_host_buffers_ms"] = median_wall_ms(torch, lambda: gb.bls12_381_g1_msm(bases, s))
    # resident bases and scalars without the precomputed table (n x 96 B of
    # bases instead of the context's 16 x n x 96 B)
    d_b = torch.from_numpy(np.ascontiguousarray(bases).view(np.int64).copy()).cuda()
    d_s = torch.from_numpy(s.view(np.int64).copy()).cuda()
    torch.cuda.synchronize()
    out["msm_2p20_resident_no_table_ms"] = median_ms(
        torch, stream, lambda: gb.g1_msm_device(d_b.data_ptr(), d_s.data_ptr(), n))
    out["msm_2p20_resident_no_table_mpts_s"] = n / out["msm_2p20_resident_no_table_ms"] / 1e3
    out["msm_no_table_device_bytes"] = n * 96
    del d_b, d_s
    # sustained throughput of back-to-back 2^20 MSMs from two lanes (two
    # host threads, one CUDA stream each): one MSM's latency-bound tail
    # overlaps the next one's sort and accumulation
    ctx2 = gb.Bls12_381G1MsmContext(bases)
    sets2 = gb.Bls12_381FrDeviceVec.upload(fr_uniform(4 * n, rng))

    def lane_worker(lane, idx):
        gb.execution_lane_set(lane)
        for i in idx:
            ctx2.device_batch(sets2, (i % 4) * n, n, 1)
        gb.execution_lane_set(0)

    lane_worker(1, range(2))
    lane_worker(2, range(2))
    rates = []
    for _ in range(3):
        ths = [threading.Thread(target=lane_worker, args=(1 + j, range(j, 10, 2))) for j in range(2)]
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        rates.append(10 * n / (time.perf_counter() - t0) / 1e6)
    out["msm_2p20_two_lanes_mpts_s"] = statistics.median(rates)
    ctx2.close()
    sets2.free()
    # 16 x NTT 2^20 forward / inverse and coset LDE 2^20 -> 2^22, resident
    log_n, count = 20, 16
    polys = fr_uniform(count << log_n, rng)
    one = np.array([0x00000001FFFFFFFE, 0x5884B7FA00034802, 0x998C4FEFECBC4FF5, 0x1824B159ACC5056F], np.uint64)
    dv = gb.Bls12_381FrDeviceVec.upload(polys)
    for name, inverse in (("ntt_2p20_x16_fwd_ms", False), ("ntt_2p20_x16_inv_ms", True)):
        out[name] = median_ms(torch, stream, lambda: dv.ntt_zeta_batch(log_n, count, inverse, one, one, one))
    # (n/2) log n Fr products per transform, 136 multiply-adds each
    ntt_madd = count * (1 << (log_n - 1)) * log_n * 136
    achieved = ntt_madd / (out["ntt_2p20_x16_fwd_ms"] * 1e-3) / 1e12
    out["roofline_ntt"] = {"bound": "imad", "unit": "Tmadd/s", "kernel": "16 x NTT 2^20, all passes",
                           "achieved": achieved, "peak": peak / 1e12, "frac": achieved / (peak / 1e12),
                           "frac_issue_ceiling": achieved / issue_ceiling_tmadd(),
                           "algorithmic": "(n/2) log2 n Fr products x 136 madd per transform"}
    del dv
    src = gb.Bls12_381FrDeviceVec.upload(polys)

    # coefficients resident -> 16 extended cosets resident: the ZETA coset
    # (reference semantics) and the coset of the generator 7
    def lde_zeta():
        h = ctypes.c_void_p()
        gb.api.check(lib.midnight_sppark_bls12_381_fr_device_coeff_to_extended_from_device_batch(
            ctypes.byref(h), src.raw, 1 << log_n, count, 22, gb.api._fr(one), gb.api._fr(one)))
        gb.Bls12_381FrDeviceVec(h).free()

    def lde_gen():
        gb.fr_device_coeff_to_extended_coset_batch(src, 1 << log_n, count, 22).free()

    out["lde_2p20_to_2p22_x16_resident_ms"] = median_ms(torch, stream, lde_zeta)
    out["lde_gen7_2p20_to_2p22_x16_resident_ms"] = median_ms(torch, stream, lde_gen)
    # butterflies (N/2) log2 N Fr products per output transform + the input factors
    lde_madd = count * ((1 << 21) * 22) * 136
    out["roofline_lde"] = {"bound": "imad", "unit": "Tmadd/s", "kernel": "16 x coset LDE 2^20 -> 2^22",
                           "achieved": lde_madd / (out["lde_2p20_to_2p22_x16_resident_ms"] * 1e-3) / 1e12,
                           "peak": peak / 1e12}
    out["roofline_lde"]["frac"] = out["roofline_lde"]["achieved"] / (peak / 1e12)
    # from pinned host memory, result resident (the host-input entry point)
    pinned = torch.empty((count << log_n, 4), dtype=torch.int64, pin_memory=True)
    host = pinned.numpy().view(np.uint64)
    host[:] = polys

    def lde_host():
        lde = gb.bls12_381_fr_device_coeff_to_extended_batch(host.reshape(count, 1 << log_n, 4), 22, one, one)
        lde.download(1)
        lde.free()

    out["lde_2p20_to_2p22_x16_host_in_ms"] = median_wall_ms(torch, lde_host)
    del src
    out.update(batched_config(gb, torch, rng))
    out.update(proof_config(gb))
    out.update(serve_config(gb))
    return out


if __name__ == "__main__":
    main()
