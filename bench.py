"""Benchmark: Monte Carlo moves per second on the 8,000-water NVT system.

Workload (the GPU configuration the metric is quoted on): 8,000 rigid
SPC/E-geometry waters (24,000 sites) in a 62.1 A cube at 298 K, Rcut 10 A,
Ewald tolerance 1e-5 (24,658 k-vectors), seeded lattice with random
orientations; single-molecule translate/rotate moves 50/50 drawn from the
reference's MT19937 stream, move sizes starting from 0.3 A / 0.3 rad with the
reference's adjustment every 1,000 moves.  One step = --moves-per-step moves
of one Markov chain per GPU, state resident in HBM.

value   : moves/s of the plain FP64 form, device time (CUDA events on the
          library's stream) summed over the timed steps, L2 flushed between
          steps; whole job over all ranks (independent replicas per GPU).
e2e     : the same metric through the public API with host buffers: each step
          draws its moves from the MT19937 stream on the host, copies the
          move records to the device and runs them (gb_mc_run), and reads
          back energies, coordinates and molecule centres.
mixed   : the mixed-precision form (FP32 pair / per-k arithmetic, FP64
          accumulators), several independent chains batched on one GPU.
serving : a stream of water jobs of mixed size through the job server
          (continuous batching), throughput and p50/p99 per-sweep latency.
gemc    : the Gibbs-ensemble configuration (2,400 + 300 LJ spheres,
          displacement / volume exchange / CBMC swap), both boxes in one
          persistent launch, FP64 and mixed forms, with the host
          restatement's rate beside it.
roofline: the dominant kernel (the persistent chain kernel) against the
          measured FP64 pipe peak of this GPU (float64 GEMM timed here).

--impl reference times the reference algorithm on the host cores instead (the
C oracle restatement, OpenMP over k-vectors, all host threads), same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

N_MOL = 8000
BOX = 62.1
RCUT = 10.0
TOL = 1e-5
TEMP = 298.0
SEED = 20260
FRAC = (0.5, 0.5, 0.0)
ADJ = 1000
SCALES = (0.3, 0.3, 0.02, 0.031415926535897934)
METRIC = ("MC moves/s, 8k-water NVT: FP64 vs mixed (|dE|<=1e-6 rel); "
          "job p50/p99 latency")
WORKLOAD = ("8000 SPC/E waters (24000 sites), L=62.1 A, Rcut 10 A, Ewald tol "
            "1e-5 (K=24658), T=298 K, translate/rotate 50/50, one chain per "
            "GPU")


def flop_per_move(K: int, na: int = 3, cand: int = 18000, incut: int = 2500):
    """Algorithmic FP64 flops of one single-molecule move.

    Reciprocal: per k-vector and per old/new atom position a dot product k.r
    (5 flops) and the charge-weighted accumulate of cos and sin (2), then the
    structure-factor update (4) and its energy (3): 49 K for a 3-site
    molecule; the 2 n_a K sine/cosine evaluations are counted apart
    (sincos_per_move).  Real space: 8 flops per candidate pair (minimum image
    and r^2) and 25 per pair inside the cutoff (LJ and erfc-screened
    Coulomb)."""
    recip = K * (2 * na * (5 + 2) + 4 + 3)
    real = cand * 8 + incut * 25
    return recip + real


def sincos_per_move(K: int, na: int = 3):
    return 2 * na * K


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
                for i, n in enumerate(names):
                    if s[4 + i].lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks(torch, dev):
    """HBM/bf16 from MEASURED_PEAKS.json; FP64/FP32 pipe peaks timed here."""
    out = {}
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            mp = json.load(f)
        out["hbm_gbs"] = mp.get("hbm_gbs")
        out["source"] = "MEASURED_PEAKS.json"
    else:
        out["hbm_gbs"] = 6800.0
        out["source"] = "fallback"
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, dt, n, reps in (("fp64_tflops", torch.float64, 4096, 3),
                              ("fp32_tflops", torch.float32, 8192, 5)):
        a = torch.randn(n, n, device=dev, dtype=dt)
        b = torch.randn(n, n, device=dev, dtype=dt)
        torch.matmul(a, b)
        torch.cuda.synchronize(dev)
        best = 1e9
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        out[name] = 2.0 * n ** 3 / best / 1e12
        del a, b
    out["pipe_peak_source"] = "float64 / float32 GEMM timed in bench.py"
    return out


# DRAM bytes (read + write) of one 1,000-move launch of each FP64 chain
# kernel on the 8,000-water workload after the L2 flush, from ncu captures
# of this command's FP64 line (dram__bytes_read.sum + dram__bytes_write.sum):
# two moves in flight 2.54 MB read, 0 written (mean of 10 launches); one
# move in flight 2.42 MB, 0 (mean of 13)
CHAIN_FP64_DRAM_BYTES_1000 = {"k_chain_fp64_pipe": 2.54e6,
                              "k_chain_fp64": 2.42e6}
SMALL = False  # --small: the 256-water, 19.7 A box (for profiler captures)


def make_system(rank: int):
    from gomc_gb300.config import SimConfig
    from gomc_gb300.systems import spce_water_box
    if SMALL:
        sysm = spce_water_box(256, 19.7, seed=SEED + rank)
        cfg = SimConfig(temperature=TEMP, rcut=9.0, tolerance=TOL)
    else:
        sysm = spce_water_box(N_MOL, BOX, seed=SEED + rank)
        cfg = SimConfig(temperature=TEMP, rcut=RCUT, tolerance=TOL)
    return sysm, cfg


def cpu_baseline(seconds: float, threads: int):
    """The oracle port on the host cores: moves/s over a bounded sample."""
    from oracle import oracle as O
    O.set_threads(threads)
    sysm, cfg = make_system(0)
    ob = O.OracleBox(sysm, cfg)
    ob.mc_init(SEED, FRAC, ADJ)
    ob.mc_set_scales(SCALES)
    step, n = 0, 0
    t0 = time.time()
    chunk = 8
    while time.time() - t0 < seconds:
        ob.mc_run(step, chunk)
        step += chunk
        n += chunk
    dt = time.time() - t0
    return {"value": n / dt, "unit": "moves/s", "cores": threads,
            "kind": "port",
            "sample": "%d single-molecule moves of the 8000-water system "
                      "(%.1f s)" % (n, dt)}


def max_over_ranks(value, dist, torch, device):
    """The largest of every rank's value (the slowest rank's time); the value
    itself in a single-process run."""
    if not dist:
        return value
    tt = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    steps, warm = args.steps, args.warmup
    from oracle import oracle as O
    O.set_threads(threads)
    sysm, cfg = make_system(0)
    ob = O.OracleBox(sysm, cfg)
    ob.mc_init(SEED, FRAC, ADJ)
    ob.mc_set_scales(SCALES)
    per_step = args.ref_moves_per_step
    step = 0
    for _ in range(warm):
        ob.mc_run(step, per_step)
        step += per_step
    t0 = time.time()
    for _ in range(steps):
        ob.mc_run(step, per_step)
        step += per_step
    dt = time.time() - t0
    v = steps * per_step / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "moves/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": warm,
        "ms_per_step": dt / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "moves_per_step": per_step,
                   "l2": "host run"},
        "cpu_baseline": {"value": v, "unit": "moves/s", "cores": threads,
                         "kind": "port",
                         "sample": "%d steps x %d moves of the same workload"
                                   % (steps, per_step)},
        "e2e": {"value": v, "unit": "moves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_mixed(args, dev, rank, world, torch, engine, barrier, dist,
              fp64_value):
    """The mixed-precision form on the same workload.

    accuracy: an FP64 chain and a mixed chain from the same seed run the same
      moves; reported are the share of identical accept decisions, the
      per-move energy-change errors and the running energy terms of the mixed
      chain against a full FP64 recompute.
    single:   one mixed chain, moves/s (device time, L2 flushed between steps).
    batched:  independent replicas of the box (seeds differ), all chains in one
      launch per step; moves/s over all chains, device time.
    e2e:      the batched run through the public API with host buffers:
      move records of every replica drawn on the host and copied in, energies
      and coordinates read back, every step.
    drift:    largest relative difference between the running energies and
      the periodic FP64 recompute (every 10,000 moves) over the run."""
    from gomc_gb300._lib import GB_FP64, GB_MIXED
    out = {}
    sysm, cfg = make_system(rank)
    n_cmp = args.mixed_compare_moves
    bf = engine.Box(sysm, cfg, device=dev, precision=GB_FP64)
    bm = engine.Box(sysm, cfg, device=dev, precision=GB_MIXED)
    for b in (bf, bm):
        b.mc_init(SEED + rank, FRAC, ADJ, scales=SCALES,
                  cluster_size=args.cluster)
    tune_single = None
    if not args.cluster:
        tune_single = bm.mc_autotune("latency")
    rf = bf.mc_run(0, n_cmp, trace=True)
    rm = bm.mc_run(0, n_cmp, trace=True)
    same = float(np.mean(rf["accepted"] == rm["accepted"]))
    sig = rm["de"] - rf["de"]
    err = np.abs(sig)
    # running-energy error the mixed chain accumulates over its accepted
    # moves (both chains take the same decisions), per term, in K
    accm = rm["accepted"].astype(bool) & rf["accepted"].astype(bool)
    acc_err = sig[accm].sum(axis=0)
    tot_f = rf["de"].sum(axis=1)
    tot_m = rm["de"].sum(axis=1)
    rel = np.abs(tot_m - tot_f) / np.maximum(np.abs(tot_f), 1e-300)
    run = bm.energy()
    st = bm.system_total()
    term_rel = {k: abs(run[i] - st[k]) / abs(st[k])
                for i, k in enumerate(["inter", "real", "recip"])}
    run_tot = float(sum(run[:5]))
    st_tot = sum(st[k] for k in ("inter", "real", "recip", "self",
                                 "correction"))
    term_rel["total"] = abs(run_tot - st_tot) / abs(st_tot)
    out["accuracy"] = {
        "moves": n_cmp, "same_decisions": same,
        "de_abs_max_K": {"inter": float(err[:, 0].max()),
                         "real": float(err[:, 1].max()),
                         "recip": float(err[:, 2].max())},
        "de_rms_K": {"inter": float(np.sqrt(np.mean(sig[:, 0] ** 2))),
                     "real": float(np.sqrt(np.mean(sig[:, 1] ** 2))),
                     "recip": float(np.sqrt(np.mean(sig[:, 2] ** 2)))},
        "accumulated_over_accepted_K": {"inter": float(acc_err[0]),
                                        "real": float(acc_err[1]),
                                        "recip": float(acc_err[2])},
        "accumulated_total_rel": float(abs(acc_err.sum()) / abs(st_tot)),
        "de_total_rel_median": float(np.median(rel)),
        "running_vs_fp64_recompute_rel": term_rel,
        "tolerance": "every running term <= 1e-6 relative of the FP64 "
                     "recompute; decisions identical"}
    layout = bm.mc_layout()
    bf.close()

    M = args.moves_per_step
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32,
                        device=dev)

    def timed(run_step, stream):
        times = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run_step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        return times

    # single mixed chain (continues from the comparison run)
    st_single = torch.cuda.ExternalStream(bm.stream_ptr(), device=dev)
    step = [n_cmp]

    def one():
        bm.mc_run(step[0], M)
        step[0] += M
    for _ in range(args.warmup):
        one()
    barrier()
    t_single = timed(one, st_single)
    bm.close()
    single = args.steps * M / sum(t_single)
    out["single"] = {"value": single, "unit": "moves/s",
                     "ms_per_step": sum(t_single) / args.steps * 1e3,
                     "us_per_move": sum(t_single) / (args.steps * M) * 1e6,
                     "ctas_per_chain": layout["ctas_per_chain"],
                     "unit_lanes": tune_single and
                     tune_single["chosen"]["unit_lanes"],
                     "autotune_us_per_move": tune_single and {
                         "%d x %d" % (t["ctas"], t["unit_lanes"]):
                         round(t["us_per_move"], 2)
                         for t in tune_single["tried"]}}

    # batched replicas, one launch per step for every chain; the cluster
    # size from the autotuner's throughput objective on the first replica
    boxes = []
    s0, c0 = make_system(rank * 1000)
    b0 = engine.Box(s0, c0, device=dev, precision=GB_MIXED)
    b0.mc_init(SEED + rank * 1000, FRAC, ADJ, scales=SCALES,
               recompute_freq=10000, cluster_size=args.cluster)
    tune_batch = None
    if not args.cluster:
        tune_batch = b0.mc_autotune("throughput")
    lay0 = b0.mc_layout()
    csize = lay0["ctas_per_chain"]
    lanes = tune_batch["chosen"]["unit_lanes"] if tune_batch else 0
    boxes.append(b0)
    B = args.mixed_chains or lay0["max_concurrent"]
    for i in range(1, B):
        s_i, c_i = make_system(rank * 1000 + i)
        b = engine.Box(s_i, c_i, device=dev, precision=GB_MIXED)
        b.mc_init(SEED + rank * 1000 + i, FRAC, ADJ, scales=SCALES,
                  recompute_freq=10000, cluster_size=csize, unit_lanes=lanes)
        boxes.append(b)
    st_batch = torch.cuda.ExternalStream(boxes[0].stream_ptr(), device=dev)
    bstep = [0]
    # every replica starts from its own seeded lattice: an untimed
    # equilibration run melts it before anything is measured, and the drift
    # windows are recorded from then on
    if args.mixed_equil_moves > 0:
        engine.mc_run_batch(boxes, 0, args.mixed_equil_moves)
        bstep[0] = args.mixed_equil_moves
    seen = [b.mc_drift()["recomputes"] for b in boxes]
    equil = {"max": {}, "recomputes": sum(seen)}
    for b in boxes:
        for k, v in b.mc_drift()["max"].items():
            equil["max"][k] = max(equil["max"].get(k, 0.0), v)
    windows = []

    def record_windows():
        for i, b in enumerate(boxes):
            d = b.mc_drift()
            if d["recomputes"] > seen[i]:
                seen[i] = d["recomputes"]
                windows.append([d["last"][k] for k in
                                ("inter", "real", "recip", "total")])

    def batch():
        engine.mc_run_batch(boxes, bstep[0], M)
        bstep[0] += M
        record_windows()
    for _ in range(args.warmup):
        batch()
    barrier()
    with ClockSampler(dev) as clk:
        t_batch = timed(batch, st_batch)
    barrier()
    t_tot = float(sum(t_batch))
    t_tot = max_over_ranks(t_tot, dist, torch, dev)
    batched = world * args.steps * M * B / t_tot
    timing = boxes[0].mc_timing(reset=True)

    # end to end through the public API with host buffers: every replica's
    # move records are drawn on the host and copied in, its energies,
    # coordinates and centres read back, every step
    e2e_t = []
    barrier()
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        engine.mc_run_batch(boxes, bstep[0], M)
        bstep[0] += M
        host = []
        for b in boxes:
            b.energy()
            host.append((b.coords(), b.com()))
        if i >= args.warmup:  # the first calls size the host staging
            e2e_t.append(time.perf_counter() - t0)
        record_windows()
    barrier()
    t_e2e = float(sum(e2e_t))
    t_e2e = max_over_ranks(t_e2e, dist, torch, dev)
    per_box = (sysm.n_atoms + sysm.n_mol) * 3 * 8
    names = ("inter", "real", "recip", "total")
    win = np.array(windows) if windows else np.zeros((0, 4))
    drift = {"max": {k: float(win[:, i].max()) if len(win) else None
                     for i, k in enumerate(names)},
             "windows": int(len(win)),
             "windows_above_1e-8": int((win[:, 3] > 1e-8).sum())
             if len(win) else 0,
             "equilibration": dict(equil, moves=args.mixed_equil_moves)}
    for b in boxes:
        b.close()
    out["batched"] = {
        "value": batched, "unit": "moves/s", "chains": B,
        "ms_per_step": sum(t_batch) / args.steps * 1e3,
        "step_ms": [round(t * 1e3, 3) for t in t_batch],
        "kernel_launches": timing["chain_launches"],
        "speedup_vs_fp64": batched / fp64_value,
        "ctas_per_chain": csize,
        "unit_lanes": lanes,
        "autotune_us_per_move": tune_batch and {
            "%d x %d" % (t["ctas"], t["unit_lanes"]): round(t["us_per_move"], 2)
            for t in tune_batch["tried"]},
        "clocks": clk.summary()}
    out["e2e"] = {"value": world * args.steps * M * B / t_e2e,
                  "unit": "moves/s",
                  "h2d_bytes_per_step": B * M * 64,
                  "d2h_bytes_per_step": B * (5 * 8 + per_box)}
    out["drift"] = dict(drift, recompute_every=10000,
                        bar="total-energy drift <= 1e-8 relative",
                        note="max over the 10,000-move windows of every "
                             "replica that ended after the untimed "
                             "equilibration (the melt of the seeded "
                             "lattice); the equilibration's own windows "
                             "under 'equilibration'")
    out["dtype"] = "f32 pair/k terms, f64 accumulators"
    return out


def run_drift(args, dev, engine):
    """One mixed chain over `--drift-moves` moves of the same workload with
    the FP64 recompute every 10,000 moves; each window's relative difference
    between the running energies and the recompute is recorded.  The chain
    starts from the seeded lattice, so the first windows cover the melt of
    the lattice (large energy changes, small |E|)."""
    from gomc_gb300._lib import GB_MIXED
    sysm, cfg = make_system(0)
    b = engine.Box(sysm, cfg, device=dev, precision=GB_MIXED)
    R = 10000
    b.mc_init(SEED + 77, FRAC, ADJ, scales=SCALES, recompute_freq=R)
    n = (args.drift_moves + R - 1) // R
    t0 = time.perf_counter()
    win = []
    for w in range(n):
        b.mc_run(w * R, R)
        d = b.mc_drift()["last"]
        win.append([d["inter"], d["real"], d["recip"], d["total"]])
    wall = time.perf_counter() - t0
    e = b.energy()
    b.close()
    win = np.array(win)
    after = win[10:] if len(win) > 10 else win[-1:]
    return {"moves": n * R, "recompute_every": R, "windows": n,
            "wall_s": wall,
            "total_max": float(win[:, 3].max()),
            "total_first_window": float(win[0, 3]),
            "total_max_after_100k_moves": float(after[:, 3].max()),
            "windows_above_1e-8": int((win[:, 3] > 1e-8).sum()),
            "term_max": {"inter": float(win[:, 0].max()),
                         "real": float(win[:, 1].max()),
                         "recip": float(win[:, 2].max())},
            "energy_end_K": float(sum(e[:5])),
            "bar": "total-energy drift <= 1e-8 relative between recomputes"}


MP_FRAC = (0.495, 0.495, 0.01)


def run_multiparticle(args, dev, engine, torch, batch_chains):
    """Config 1 with the MultiParticle move in the mix (translate / rotate /
    MultiParticle 0.495 / 0.495 / 0.01): moves/s of the FP64 chain, of one
    mixed chain and of the batched mixed replicas, with the device time per
    move of each move type (chain segments, MultiParticle kernel
    sequences: BoxForce, the full structure factor, BoxForceReciprocal)."""
    from gomc_gb300._lib import GB_FP64, GB_MIXED
    M = args.moves_per_step
    steps = max(3, args.steps // 2)
    out = {"workload": WORKLOAD.replace("translate/rotate 50/50",
                                        "translate/rotate/MultiParticle "
                                        "0.495/0.495/0.01"),
           "moves_per_step": M, "steps": steps}

    def timed_run(boxes, stream, batched):
        for b in boxes:
            b.mc_timing(reset=True)
        step = 0
        for _ in range(args.warmup):
            if batched:
                engine.mc_run_batch(boxes, step, M)
            else:
                boxes[0].mc_run(step, M)
            step += M
        for b in boxes:
            b.mc_timing(reset=True)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(steps):
            if batched:
                engine.mc_run_batch(boxes, step, M)
            else:
                boxes[0].mc_run(step, M)
            step += M
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        tm = [b.mc_timing() for b in boxes]
        chain_ms = sum(t["chain_ms"] for t in tm)
        mp_ms = sum(t["mp_ms"] for t in tm)
        chain_moves = sum(t["chain_moves"] for t in tm)
        mp_moves = sum(t["mp_moves"] for t in tm)
        total = steps * M * len(boxes)
        return {"value": total / wall, "unit": "moves/s",
                "wall_s": wall, "replicas": len(boxes),
                "single_molecule_us_per_move":
                    chain_ms * 1e3 / max(chain_moves, 1),
                "multiparticle_ms_per_move": mp_ms / max(mp_moves, 1),
                "multiparticle_moves": mp_moves,
                "device_ms": {"chains": chain_ms, "multiparticle": mp_ms}}

    sysm, cfg = make_system(0)
    box = engine.Box(sysm, cfg, device=dev, precision=GB_FP64)
    box.mc_init(SEED + 5, MP_FRAC, ADJ, scales=SCALES)
    out["fp64"] = timed_run([box], None, False)
    box.close()
    box = engine.Box(sysm, cfg, device=dev, precision=GB_MIXED)
    box.mc_init(SEED + 5, MP_FRAC, ADJ, scales=SCALES, recompute_freq=10000,
                cluster_size=args.cluster or 16)
    out["mixed_single"] = timed_run([box], None, False)
    box.close()
    boxes = []
    for i in range(batch_chains):
        s_i, c_i = make_system(2000 + i)
        b = engine.Box(s_i, c_i, device=dev, precision=GB_MIXED)
        b.mc_init(SEED + 2000 + i, MP_FRAC, ADJ, scales=SCALES,
                  recompute_freq=10000, cluster_size=args.cluster or 8)
        boxes.append(b)
    out["mixed_batched"] = timed_run(boxes, None, True)
    for b in boxes:
        b.close()
    out["note"] = ("wall-clock moves/s (host move drawing and the "
                   "MultiParticle kernel sequences' synchronisations "
                   "included); per-type device times from CUDA events on "
                   "the boxes' streams")
    return out


GEMC_CFG = dict(temperature=150.0, rcut=12.0, eps=148.0, sigma=3.73,
                frac=(0.8, 0.01, 0.19), adj=100, cbmc_first=10, seed=3333)


def gemc_boxes():
    """The Gibbs-ensemble configuration: 2,400 LJ spheres in a 40 A box and
    300 in a 90 A box at seeded non-overlapping random positions."""
    from gomc_gb300.systems import lj_sphere_box
    s0 = lj_sphere_box(2400, 40.0, seed=31, epsilon=GEMC_CFG["eps"],
                       sigma=GEMC_CFG["sigma"], min_sep=2.4, name="LJ")
    s1 = lj_sphere_box(300, 90.0, seed=32, epsilon=GEMC_CFG["eps"],
                       sigma=GEMC_CFG["sigma"], min_sep=3.5, name="LJ")
    return s0, s1


def run_gemc(args, dev, engine, torch):
    """Gibbs-ensemble NVT of LJ spheres (both boxes in one persistent
    launch): moves/s of the FP64 and mixed forms, device time per launch of
    --gemc-moves moves, L2 flushed between launches; the oracle's host
    restatement of the same run as the CPU baseline."""
    from gomc_gb300._lib import GB_FP64, GB_MIXED
    s0, s1 = gemc_boxes()
    g = GEMC_CFG
    M = args.gemc_moves
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32,
                        device=dev)
    out = {"workload": "GEMC NVT, LJ spheres eps/kB 148 K, sigma 3.73 A, "
                       "Rcut 12 A, T 150 K: 2,400 in 40 A + 300 in 90 A, "
                       "displacement / volume / swap 0.8 / 0.01 / 0.19, "
                       "10 CBMC trials, %d moves per launch" % M}
    runs = {}
    for name, prec in (("fp64", GB_FP64), ("mixed", GB_MIXED)):
        gm = engine.Gemc(s0.pos, s1.pos, s0.box, s1.box, g["eps"], g["sigma"],
                         12.0, g["temperature"], g["rcut"], g["seed"],
                         g["frac"], g["adj"], g["cbmc_first"], precision=prec,
                         device=dev)
        for _ in range(args.warmup):
            gm.run(M)
        # where one launch's time goes (an untimed launch with the phase
        # clocks of the cluster's first CTA)
        gm.profile(True)
        gm.run(M)
        phases = gm.profile(False)
        ms = []
        kinds = np.zeros(3, np.int64)
        acc = np.zeros(3, np.int64)
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            r = gm.run(M, trace=True)
            ms.append(gm.state()["last_ms"])
            for i, k in enumerate((0, 13, 10)):
                sel = r["kind"] == k
                kinds[i] += int(sel.sum())
                acc[i] += int(r["accepted"][sel].sum())
        st = gm.state()
        tot = gm.system_total()
        runs[name] = {
            "value": args.steps * M / (sum(ms) / 1e3), "unit": "moves/s",
            "us_per_move": sum(ms) * 1e3 / (args.steps * M),
            "launch_ms": [round(v, 3) for v in ms],
            "moves_by_kind": {"displacement": int(kinds[0]),
                              "volume": int(kinds[1]),
                              "transfer": int(kinds[2])},
            "accepted_by_kind": {"displacement": int(acc[0]),
                                 "volume": int(acc[1]),
                                 "transfer": int(acc[2])},
            "molecules_box0": st["n0"],
            "phase_us_per_move": phases,
            "running_vs_recompute_rel": [
                float(abs(st["energy"][b] - tot[b]) / max(abs(tot[b]), 1.0))
                for b in range(2)]}
        gm.close()
    out.update(runs)
    out["mixed_speedup_vs_fp64"] = runs["mixed"]["value"] / runs["fp64"]["value"]
    if not args.no_cpu:
        from oracle import oracle as O
        ob = O.OracleGemc(s0.pos, s1.pos, s0.box, s1.box, g["eps"],
                          g["sigma"], 12.0, g["temperature"], g["rcut"],
                          g["seed"], g["frac"], g["adj"], g["cbmc_first"])
        t0 = time.time()
        done = 0
        while time.time() - t0 < args.gemc_cpu_seconds:
            ob.run(done, 500)
            done += 500
        dt = time.time() - t0
        out["cpu_baseline"] = {"value": done / dt, "unit": "moves/s",
                               "cores": 1, "kind": "port",
                               "sample": "first %d moves of the same run "
                                         "(%.1f s)" % (done, dt)}
    return out


def run_serving(args, dev):
    """Serving stream on one GPU, scaled down from 256 jobs x 100 sweeps
    (the longest job alone then needs 2 x 20,000 sequential moves, the tail):
    jobs of N waters, N log-uniform in [500, 20000] at 1 g/cm^3 (SPC/E, Rcut
    9 A, Ewald tol 1e-5, T = 298 K), seeded lattices, Poisson arrivals at a
    seeded rate, each asking for --serve-sweeps sweeps (1 sweep = N moves),
    mixed form with an FP64 recompute every 10,000 moves; jobs are admitted by
    device memory and chain slots and batched per round while they run."""
    from gomc_gb300 import serving
    from gomc_gb300.config import SimConfig
    from gomc_gb300.systems import spce_water_box, water_box_length
    rng = np.random.default_rng(SEED)
    J, sweeps = args.serve_jobs, args.serve_sweeps
    sizes = np.exp(rng.uniform(np.log(500), np.log(20000), J)).astype(int)
    gaps = rng.exponential(1.0 / args.serve_rate, J)
    cfg = SimConfig(temperature=TEMP, rcut=9.0, tolerance=TOL)
    systems = [spce_water_box(int(n), water_box_length(int(n)), seed=SEED + i)
               for i, n in enumerate(sizes)]
    srv = serving.Server(device=dev, quantum=args.serve_quantum)
    srv.start()
    t0 = time.perf_counter()
    jids = []
    for i, (s, n) in enumerate(zip(systems, sizes)):
        target = t0 + float(np.sum(gaps[:i + 1]))
        delay = target - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        jids.append(srv.submit(s, cfg, seed=SEED + i, nsteps=int(n) * sweeps,
                               scales=SCALES, adj_steps=ADJ,
                               recompute_freq=10000))
    srv.drain(timeout_s=args.serve_timeout)
    st = srv.stats()
    # per size class (quartiles of N): queueing (submission to admission)
    # and the time per sweep once admitted, which grows with N (a sweep is
    # N sequential moves of one chain)
    jobs = [srv.job(j) for j in jids]
    srv.close()
    edges = np.quantile(sizes, [0.0, 0.25, 0.5, 0.75, 1.0])
    by_size = []
    for q in range(4):
        sel = [k for k in range(J) if (sizes[k] >= edges[q]) and
               (sizes[k] < edges[q + 1] or q == 3)]
        if not sel:
            continue
        wait = np.array([jobs[k]["t_admit"] - jobs[k]["t_submit"]
                         for k in sel])
        run = np.array([(jobs[k]["t_done"] - jobs[k]["t_admit"]) / sweeps
                        for k in sel])
        by_size.append({"waters": [int(sizes[sel].min()), int(sizes[sel].max())],
                        "jobs": len(sel),
                        "queue_s": {"p50": float(np.percentile(wait, 50)),
                                    "p99": float(np.percentile(wait, 99))},
                        "s_per_sweep_admitted": {
                            "p50": float(np.percentile(run, 50)),
                            "p99": float(np.percentile(run, 99))}})
    return {
        "workload": "%d water jobs, N log-uniform in [500, 20000] (sum %d "
                    "molecules), %d sweeps each, Poisson arrivals at %.1f "
                    "jobs/s, base quantum %d moves per round"
                    % (J, int(sizes.sum()), sweeps, args.serve_rate,
                       args.serve_quantum),
        "moves_per_s": st["moves_per_s"], "moves": st["moves"],
        "wall_s": st["wall_s"],
        "sweep_latency_ms": {"p50": st["sweep_p50_ms"],
                             "p99": st["sweep_p99_ms"]},
        "job_latency_s": {"p50": st["job_p50_s"], "p99": st["job_p99_s"]},
        "rounds": st["rounds"], "mean_resident_jobs": st["mean_resident"],
        "occupancy": {k: st[k] for k in ("mean_admitted", "mean_in_round",
                                         "cta_slot_frac", "smem_frac",
                                         "mean_queued", "stops_mem",
                                         "stops_smem", "stops_ctas",
                                         "launch_balance", "round_gap_s")},
        "helper_busy_s": st["helper_busy_s"], "round_busy_s": st["round_busy_s"],
        "jobs_done": st["jobs_done"], "by_size_quartile": by_size}


def run_gb300(args, rank, world):
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    from gomc_gb300 import engine
    engine.lib(build_if_missing=True)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    sysm, cfg = make_system(rank)
    box = engine.Box(sysm, cfg, device=dev)
    K, kmax = box.num_kvectors()
    box.mc_init(SEED + rank, FRAC, ADJ, scales=SCALES)
    shape = box.mc_shape()
    chain_kernel = ("k_chain_fp64_pipe" if shape["moves_in_flight"] == 2
                    else "k_chain_fp64")
    stream = torch.cuda.ExternalStream(box.stream_ptr(), device=dev)
    M = args.moves_per_step
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32,
                        device=dev)
    step = 0
    for _ in range(args.warmup):
        box.mc_run(step, M)
        step += M
    box.mc_timing(reset=True)
    times = []
    barrier()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            box.mc_run(step, M)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            step += M
    barrier()
    timing = box.mc_timing(reset=True)
    # where a move's time goes: the chain's phase clocks over 2,000 further
    # moves (outside the timed steps)
    box.mc_profile(enable=True)
    box.mc_run(step, 2000)
    step += 2000
    pr = box.mc_profile(enable=False)
    phase_us = {who: {k: v / max(pr["moves"][i], 1)
                      for k, v in pr[who].items()}
                for i, who in enumerate(("cta0", "leader"))}
    phase_us["cta0"]["context_written_after_phase_a"] = (
        pr["cta0_context_written_after_phase_a"] / max(pr["moves"][0], 1))
    t_total = float(sum(times))
    t_total = max_over_ranks(t_total, dist, torch, dev)
    value = world * args.steps * M / t_total

    # end to end through the public API with host buffers: each step's
    # inputs are its move records (molecule, kind, displacement and
    # acceptance draws of the reference's MT19937 stream, drawn on the host
    # and copied to the device, 64 B per move); its results, the running
    # energies, coordinates and molecule centres, are read back
    e2e_times = []
    barrier()
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        box.mc_run(step, M)
        e = box.energy()
        xyz = box.coords()
        com = box.com()
        if i >= args.warmup:  # the first calls size the host staging
            e2e_times.append(time.perf_counter() - t0)
        step += M
    barrier()
    t_e2e = float(sum(e2e_times))
    t_e2e = max_over_ranks(t_e2e, dist, torch, dev)
    e2e_value = world * args.steps * M / t_e2e
    h2d = M * 64
    d2h = 5 * 8 + (sysm.n_atoms + sysm.n_mol) * 3 * 8

    # correctness of the running energies after the timed steps
    e_run = box.energy()
    st = box.system_total()
    drift = {k: abs(e_run[i] - st[k]) / abs(st[k])
             for i, k in enumerate(["inter", "real", "recip"])}

    mixed = None
    if not args.no_mixed:
        box.close()
        mixed = run_mixed(args, dev, rank, world, torch, engine, barrier, dist,
                          value)

    serving_stats = None
    if not args.no_serving and rank == 0:
        serving_stats = run_serving(args, dev)
    gemc_stats = None
    if not args.no_gemc and rank == 0:
        gemc_stats = run_gemc(args, dev, engine, torch)
    mp_stats = None
    if not args.no_mp and rank == 0:
        mp_stats = run_multiparticle(args, dev, engine, torch,
                                     args.mp_chains)
    drift_run = None
    if args.drift_moves > 0 and rank == 0:
        drift_run = run_drift(args, dev, engine)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # the pipe peaks for the roofline, timed after every timed line: the
    # chain kernel of a box set up after these GEMMs ran about 5 % slower
    # (8.51 against 8.12 ms per 1,000-move launch on one GB300; the cause
    # was not isolated)
    peaks = measured_peaks(torch, dev)
    # per chain launch: k_fill_u64 (partial slots), the chain kernel, and
    # the grid rebuild k_cell_scatter + k_cell_sort_fill
    launches = 4 * timing["chain_launches"] + 10 * timing["mp_moves"]
    kern_ms = timing["chain_ms"] / max(timing["chain_launches"], 1)
    moves_per_launch = timing["chain_moves"] / max(timing["chain_launches"], 1)
    fl = flop_per_move(K)
    achieved = fl * moves_per_launch / (kern_ms / 1e3) / 1e12
    # DRAM bytes of one 1,000-move launch from an ncu capture of this
    # command; other move counts: null
    traffic = (CHAIN_FP64_DRAM_BYTES_1000.get(chain_kernel)
               if not SMALL and round(moves_per_launch) == 1000 else None)
    roof = {"bound": "fp64", "achieved": achieved,
            "peak": peaks["fp64_tflops"], "unit": "TFLOP/s",
            "frac": achieved / peaks["fp64_tflops"], "traffic": traffic,
            "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + "
                            "dram__bytes_write.sum)",
            "kernel": chain_kernel,
            "per_unit": "%.3g FP64 flop per move (%d k-vectors), plus %d "
                        "sin/cos evaluations" % (fl, K, sincos_per_move(K)),
            "peak_source": peaks["pipe_peak_source"],
            "hbm_peak_gbs": peaks["hbm_gbs"], "hbm_peak_source": peaks["source"]}
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(args.cpu_seconds, os.cpu_count() or 1)
    line = {
        "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "moves_per_step": M,
                   "l2": "flushed between steps (512 MB write)",
                   "precision": "FP64 plain form", "k_vectors": K,
                   "chain": {"kernel": chain_kernel,
                             "grid_ctas": shape["ctas"],
                             "moves_in_flight": shape["moves_in_flight"]}},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "moves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "running_vs_recompute_rel": drift,
        "step_ms": [round(t * 1e3, 3) for t in times],
        "e2e_step_ms": [round(t * 1e3, 3) for t in e2e_times],
        "chain_kernel_ms_per_launch": kern_ms,
        "chain_phase_us_per_move": phase_us,
        "mixed": mixed,
        "serving": serving_stats,
        "gemc": gemc_stats,
        "multiparticle": mp_stats,
    }
    if drift_run:
        line["mixed_drift_run"] = drift_run
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--moves-per-step", type=int, default=1000)
    ap.add_argument("--ref-moves-per-step", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--mixed-chains", type=int, default=0,
                    help="replicas in the batched mixed run (0: as many as "
                         "the GPU holds at once)")
    ap.add_argument("--cluster", type=int, default=0,
                    help="CTAs per mixed chain (0: autotuned)")
    ap.add_argument("--mixed-compare-moves", type=int, default=10000)
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-jobs", type=int, default=96)
    ap.add_argument("--serve-sweeps", type=int, default=2)
    ap.add_argument("--serve-rate", type=float, default=64.0,
                    help="job arrivals per second (Poisson)")
    ap.add_argument("--serve-quantum", type=int, default=1000)
    ap.add_argument("--serve-timeout", type=float, default=600.0,
                    help="seconds the serving stream may take to drain")
    ap.add_argument("--mixed-equil-moves", type=int, default=20000,
                    help="untimed moves of every batched replica before "
                         "the measured steps")
    ap.add_argument("--drift-moves", type=int, default=1000000,
                    help="also run one mixed chain this many moves and "
                         "report the drift of every 10,000-move window")
    ap.add_argument("--no-gemc", action="store_true")
    ap.add_argument("--no-mp", action="store_true",
                    help="skip the line with MultiParticle moves in the mix")
    ap.add_argument("--mp-chains", type=int, default=16,
                    help="replicas of the batched mixed MultiParticle run")
    ap.add_argument("--gemc-moves", type=int, default=20000,
                    help="moves per launch of the Gibbs-ensemble line")
    ap.add_argument("--gemc-cpu-seconds", type=float, default=5.0)
    ap.add_argument("--small", action="store_true",
                    help="256-water box instead of the 8000-water workload")
    args = ap.parse_args()
    global SMALL
    SMALL = args.small
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gb300(args, rank, world)


if __name__ == "__main__":
    main()
