#!/usr/bin/env python
"""Benchmark of the GB300 sampling path: bead-moves/s on the config-1 system
(1 asymmetric-top SO2-like rotor + 64 para-H2, T = 0.37 K, P = 1024
translational / Q = 256 rotational slices, 200x60x60 rotor-atom potential,
61x121x121 rotational density), synthetic seeded tables.

A step is one pass of the reference schedule (mc_main.cc:348-381): per type
one centroid move per atom, N*P bisections of 2^L - 1 beads, and P sweeps of
the Q rotational slices.  Bead-moves per pass are counted as the reference
schedule counts them.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference path (the oracle
port, OpenMP over the host cores, the reference schedule) on a bounded sample
of the same workload; the reference's compiled objects are x86 builds of
this container and cannot run on the Arm GPU host.
Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path does not shard); value is all ranks' bead-moves over the slowest
rank's time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

# independent chains run on their own streams: give the process enough
# hardware work queues that they do not share them (read at CUDA start-up)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "moribs-pimc_gb300")
for p in (PKG, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "bead-moves/s on 1 GB300: plain vs surrogate+batched, at matched <E> error"
# DRAM traffic per launch from ncu captures of the bench's own workload, and
# the FP64 pipe's activity in the same capture:
# {(kind, mixed): {"bytes": ..., "fp64_pipe": ..., "commit": ...}}, kind 2 = the rotational sweeps
TRAFFIC_CAPTURE = {(2, False): {"bytes": 6191872 + 62720, "fp64_pipe": 0.5853, "commit": "951d278"}}
UNIT = "bead-moves/s"
WORKLOAD = "config1: 1 asymmetric-top SO2 + 64 pH2, T=0.37 K, P=1024, Q=256, L=3, plain method"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-companion", action="store_true", help="skip the other precision's measurement")
    ap.add_argument("--no-batched", action="store_true", help="skip the config-2 replica-batch measurement")
    ap.add_argument("--batched-replicas", type=int, default=4096)
    ap.add_argument("--no-tables", action="store_true", help="skip the propagator-table generator measurement")
    ap.add_argument("--no-worm", action="store_true", help="skip the worm-algorithm pass measurement")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the surrogate / delayed-acceptance measurement")
    ap.add_argument("--worm-replicas", type=int, default=32, help="independent worm chains run at once")
    ap.add_argument("--se-mode", default="default", choices=["quick", "default", "full"],
                    help="matched-SE measurement: short series (quick), the bench line's (default), or more "
                         "sampled plain replicas and the half-sweep dimer arm (full)")
    ap.add_argument("--no-matched-se", action="store_true", help="skip the matched <E> SE measurement")
    ap.add_argument("--no-precision-error", action="store_true", help="skip the FP32-vs-FP64 per-replica comparison")
    ap.add_argument("--da-replicas", type=int, default=32, help="independent dimer systems swept at once")
    ap.add_argument("--only", default=None,
                    choices=["tables", "worm", "surrogate", "matched_se", "water_chains", "config_table",
                             "fp64_pipe"],
                    help="run one companion measurement alone on cuda:0 and print its JSON (for profiling)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def dist_init(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend="gloo")
    return dist


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def workload(rank=0):
    import workloads as W
    return W.config1(seed=4321 + 17 * rank)


def host_cpu():
    try:
        model = ""
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        return model
    except OSError:
        return ""


def cpu_baseline(w, seconds, nthreads):
    """The oracle restatement of the reference schedule on the host cores, in
    its timing build (the reference's -Ofast -march=native flags): time
    slices 0, 1, ... (centroid moves at slice 0) until `seconds` pass."""
    import oracle as O
    o = O.Oracle(w, timing=True)
    done_t = 0
    bm = 0.0
    t0 = time.perf_counter()
    chunk = 8
    while True:
        st, b = o.run_steps(done_t, chunk, seed=99, nthreads=nthreads)
        if st != 0:
            raise RuntimeError("oracle run_steps failed: %d" % st)
        bm += b
        done_t += chunk
        el = time.perf_counter() - t0
        if el >= seconds or done_t >= w.nslices:
            break
    rate = bm / el
    sample = ("oracle port of the reference schedule (%s), time slices 0..%d of one pass of %s "
              "(%.3g bead-moves, %.1f s, %d threads)" % (O.timing_flags(), done_t - 1, WORKLOAD.split(":")[0], bm,
                                                          el, nthreads))
    return rate, sample


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev):
        self.dev = dev
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
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
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    except (OSError, ValueError):
        return 6800.0, "fallback"


def bf16_peak():
    """The measured dense bf16 rate (TFLOP/s, burst), else the fallback."""
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        for k in ("bf16_tflops", "bf16_tflops_burst"):
            if k in d:
                return float(d[k]), "measured (MEASURED_PEAKS.json %s)" % k
    except Exception:
        pass
    return 1900.0, "fallback"


def pair_bytes(mixed):
    """Compulsory bytes of one pair evaluation: the partner bead and 4 table
    words (FP64: 24 + 32 B; FP32 path: 12 + 16 B)."""
    return (12 + 16) if mixed else (24 + 32)


def rotation_pass_bytes(w, mixed):
    """Compulsory bytes of the P rotational sweeps of one pass (2P half-sweeps
    of Q/2 slice moves): per slice move and rotor, 2*R*(N-1) rotor-atom pair
    evaluations, 4 rotational density lookups of 4 corners, the 3
    neighbouring orientations (3 x 24 B) and the rotor's R beads."""
    P, Q = w.nslices, w.nrotslices
    R = P // Q
    na = w.natoms
    nr = sum(t["numb"] for t in w.types if t["molecule"] != 0)
    corner = 4 if mixed else 8
    per_slice = nr * (2 * R * (na - 1) * pair_bytes(mixed) + 4 * 4 * corner + 3 * 24 + R * 24)
    return P * Q * per_slice


def bisection_pass_bytes(w, mixed):
    """Compulsory bytes of the bisection blocks of one pass: per type N*P
    window moves, each with 2(M-1) slice energies over N-1 partners (all
    levels evaluated)."""
    tot = 0
    for t in w.types:
        M = 1 << t["levels"]
        tot += t["numb"] * w.nslices * 2 * (M - 1) * (w.natoms - 1) * pair_bytes(mixed)
    return tot


def centroid_pass_bytes(w, mixed):
    """Each centroid move sums the displaced and the current path of one atom
    against all partners over all P slices."""
    return w.natoms * 2 * w.nslices * (w.natoms - 1) * pair_bytes(mixed)


# FP64 operations per evaluation, counted in the reference's source (an add,
# multiply, divide, square root or transcendental call counts one; the
# library calls' own instructions are not counted): vcord + vcalc
# (vcord.f:1-98, vcalc.f:1-65) 53, including PotRotE3D's add; rotden's
# deleul + rotpro (rotden.f:1-163, rotpro_sub.f:1-64) 80; the Metropolis
# ratio and test of MCRot3Dstep (mc_piqmc.cc:1129-1178) 12.
FLOP_VCORD, FLOP_ROTDEN, FLOP_ACCEPT = 53, 80, 12


def rotation_pass_flops(w):
    """Useful FP64 operations of the P rotational sweeps of one pass of a
    nonlinear rotor: per slice move and rotor 2 R (N - 1) vcord terms (old
    and new orientation, as the reference evaluates them), 4 rotden lookups
    and the accept."""
    P, Q = w.nslices, w.nrotslices
    R = P // Q
    nr = sum(t["numb"] for t in w.types if t["molecule"] != 0)
    per = 2 * R * (w.natoms - 1) * FLOP_VCORD + 4 * FLOP_ROTDEN + FLOP_ACCEPT
    return P * Q * nr * per


def timed_passes(s, seed, steps, flush, ext, dist):
    """K passes, each bracketed by CUDA events on the library's stream, with
    an L2 flush (256 MiB write) before each outside the events; returns the
    max over ranks of the summed event time in ms."""
    import torch
    evs = []
    with torch.cuda.stream(ext):
        for k in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            s.run_passes(1, seed)
            e1.record(ext)
            evs.append((e0, e1))
    s.synchronize()
    torch.cuda.synchronize()
    return reduce_max(dist, sum(a.elapsed_time(b) for a, b in evs))


def e2e_passes(s, w, seed, steps, dist):
    """The same metric through the C ABI with host buffers: per step the path
    goes in from pinned host memory, one pass runs, and the path and the
    estimators come back."""
    import numpy as np
    import torch
    import pimc_gb300 as G
    c, a, co, p = s.get_state()
    pin_c = torch.from_numpy(c).pin_memory().numpy()
    pin_a = torch.from_numpy(a).pin_memory().numpy()
    out_c = torch.empty(c.shape, dtype=torch.float64).pin_memory().numpy()
    out_a = torch.empty(a.shape, dtype=torch.float64).pin_memory().numpy()
    out_co = torch.empty(c.shape, dtype=torch.float64).pin_memory().numpy()
    out_p = np.zeros(w.natoms, np.int32)
    est = np.zeros(5)
    barrier(dist)
    t0 = time.perf_counter()
    for k in range(steps):
        G._chk(s.L.pimc_set_state(s.h, G.dptr(pin_c), G.dptr(pin_a), G.iptr(p)), "set_state")
        s.run_passes(1, seed)
        G._chk(s.L.pimc_get_state(s.h, G.dptr(out_c), G.dptr(out_a), G.dptr(out_co), G.iptr(out_p)), "get_state")
        G._chk(s.L.pimc_estimators(s.h, G.dptr(est)), "estimators")
        pin_c[...] = out_c
        pin_a[...] = out_a
    e2e_s = reduce_max(dist, time.perf_counter() - t0)
    return {"value": s.bead_moves_per_pass() * steps * (dist.get_world_size() if dist else 1) / e2e_s, "unit": UNIT,
            "h2d_bytes_per_step": int(pin_c.nbytes + pin_a.nbytes + p.nbytes),
            "d2h_bytes_per_step": int(out_c.nbytes + out_a.nbytes + out_co.nbytes + out_p.nbytes + est.nbytes),
            "steps": steps, "path": "pimc_set_state + pimc_run_passes(1) + pimc_get_state + pimc_estimators"}


def run_gb300(args, rank, local, world, dist):
    import numpy as np
    import torch
    import pimc_gb300 as G

    torch.cuda.set_device(local)
    w = workload(rank)
    mixed = args.precision == "mixed"
    s = G.Sampler(w, device=local, mixed=mixed)
    bm_pass = s.bead_moves_per_pass()
    seed = 1000 + rank
    ext = torch.cuda.ExternalStream(s.stream(), device=torch.device("cuda", local))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > 129 MB L2
    # warm-up: graph instantiation + W passes
    s.run_passes(args.warmup, seed)
    s.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    l0 = s.launch_count()
    total_ms = timed_passes(s, seed, args.steps, flush, ext, dist)
    l1 = s.launch_count()
    ck = clocks.stop()
    value = bm_pass * args.steps * world / (total_ms / 1e3)
    tot, acc = s.counters()

    # ---- roofline of the dominant kernel from a live per-kind profile
    ms, nl = s.profile_pass(seed + 7)
    kinds = ["centroid", "bisection", "rotation"]
    dom = int(np.argmax(ms))
    bytes_pass = [centroid_pass_bytes(w, mixed), bisection_pass_bytes(w, mixed), rotation_pass_bytes(w, mixed)]
    knames = ["k_mol_pairs (centroid partner sums)", "k_bisect_block (bisection block, one CTA per window)",
              "k_rot_slices (persistent rotational sweeps, one CTA per slice)"]
    kname = knames[dom]
    bytes_launch = bytes_pass[dom] / max(1, nl[dom])
    per_launch_ms = ms[dom] / max(1, nl[dom])
    achieved = bytes_launch / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    # DRAM bytes per launch of the same kernel, workload and launch shape from
    # one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum), taken at
    # the commit named beside it; None for a kernel or precision not captured
    traffic = TRAFFIC_CAPTURE.get((dom, mixed))
    fp64_peak = G.fp64_peak(local)
    fp64_rate = rotation_pass_flops(w) / (ms[2] / 1e3) / 1e9 if ms[2] > 0 else None
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic["bytes"] if traffic else None,
                "traffic_source": ("ncu capture of this kernel and workload at commit %s" % traffic["commit"])
                if traffic else None,
                "fp64": {"kernel": knames[2], "useful_gflops": round(fp64_rate, 2) if fp64_rate else None,
                         "peak_gflops": round(fp64_peak, 1), "peak_source": "measured in this run (pimc_fp64_peak: "
                         "independent FP64 FMA chains, CUDA events)",
                         "fp64_frac": round(fp64_rate / fp64_peak, 4) if fp64_rate else None,
                         "fp64_pipe_active_frac": traffic.get("fp64_pipe") if traffic else None,
                         "flop_model": "per slice move 2R(N-1) vcord x %d + 4 rotden x %d + %d (reference source "
                                       "operations)" % (FLOP_VCORD, FLOP_ROTDEN, FLOP_ACCEPT)},
                "kernel": kname, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "per_launch_us": round(per_launch_ms * 1e3, 3), "algorithmic_bytes_per_launch": int(bytes_launch),
                "pass_ms_by_kind": {k: round(v, 3) for k, v in zip(kinds, ms)},
                "launches_by_kind": {k: int(v) for k, v in zip(kinds, nl)}}

    # ---- end to end through the C ABI with host buffers
    e2e = e2e_passes(s, w, seed + 11, args.e2e_steps, dist)
    s.close()

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if not mixed else "f32+f64",
            "data": "synthetic (seeded tables and paths of the config shapes; no dataset)",
            "config": {"workload": WORKLOAD, "bead_moves_per_pass": bm_pass, "precision": args.precision,
                       "replicas": world, "l2": "flushed between timed steps (256 MiB write)",
                       "accept_ratios": {"pH2 centroid": acc[0] / max(1, tot[0]), "pH2 bisection": acc[1] / max(1, tot[1]),
                                         "rotor bisection": acc[4] / max(1, tot[4]), "rotation": acc[5] / max(1, tot[5])}},
            "roofline": roofline, "e2e": e2e, "gpu_launches": int(l1 - l0), "clocks": ck}

    # ---- the other precision of the same path, measured the same way
    if not args.no_companion:
        other = "fp64" if mixed else "mixed"
        s2 = G.Sampler(w, device=local, mixed=not mixed)
        ext2 = torch.cuda.ExternalStream(s2.stream(), device=torch.device("cuda", local))
        s2.run_passes(args.warmup, seed)
        s2.synchronize()
        barrier(dist)
        t2 = timed_passes(s2, seed, args.steps, flush, ext2, dist)
        ms2, _ = s2.profile_pass(seed + 7)
        e2 = e2e_passes(s2, w, seed + 11, args.e2e_steps, dist)
        s2.close()
        line["companion"] = {
            "precision": other, "dtype": "f32+f64" if other == "mixed" else "f64",
            "what": ("FP32 table interpolation and partner sums, FP64 action differences, exponents, "
                     "accept tests and path" if other == "mixed" else "all arithmetic in FP64 as the reference"),
            "value": bm_pass * args.steps * world / (t2 / 1e3), "unit": UNIT, "ms_per_step": t2 / args.steps,
            "pass_ms_by_kind": {k: round(v, 3) for k, v in zip(kinds, ms2)}, "e2e": e2["value"]}
    if not args.no_batched:
        line["batched"] = run_batched(args, local, dist)
    return line, w


def run_batched(args, local, dist):
    """Config 2, the replica batch: independent replicas of the config-0
    family -- N_He uniform in 1..64, P in {64, 128, 256, 512}, Q = P/4, T
    uniform in 0.3-2.0 K, seeded -- in one persistent graph-captured launch
    per pass, FP32 tables with FP64 action differences; warps per CTA from
    the autotuner.  Timed like the main line: CUDA events around each pass,
    L2 flushed between passes."""
    import torch
    import pimc_gb300 as G
    import workloads as W
    ws = W.config2(n=args.batched_replicas, seed=2024 + 7 * (dist.get_rank() if dist else 0))
    b = G.Batch(ws, device=local, mixed=True)
    shape, tune_ms = b.autotune(77)
    ext = torch.cuda.ExternalStream(b.stream(), device=torch.device("cuda", local))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    b.run_passes(1, 78)
    b.synchronize()
    barrier(dist)
    steps = 2
    evs = []
    with torch.cuda.stream(ext):
        for k in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            b.run_passes(1, 78)
            e1.record(ext)
            evs.append((e0, e1))
    b.synchronize()
    torch.cuda.synchronize()
    total_ms = reduce_max(dist, sum(a.elapsed_time(c) for a, c in evs))
    bm = b.bead_moves_per_pass()
    world = dist.get_world_size() if dist else 1
    tot, acc = b.counters()
    out = {"workload": "config2: %d replicas of 1 CO2-like linear rotor + N He (N in 1..64, P in "
                       "{64,128,256,512}, Q=P/4, T in 0.3-2.0 K)" % len(ws),
           "value": bm * steps * world / (total_ms / 1e3), "unit": UNIT, "ms_per_pass": total_ms / steps,
           "steps": steps, "bead_moves_per_pass": bm, "precision": "mixed", "dtype": "f32+f64",
           "shape": {"warps_per_cta": shape[0], "ctas_per_sm_bound": shape[1]},
           "autotune_ms_per_pass": {"%dx%d" % sh: t for sh, t in zip(((2, 2), (4, 2), (8, 2), (4, 3), (8, 3), (2, 3)),
                                                                         [float(x) for x in tune_ms])},
           "accept_ratios": {"He bisection": acc[1] / max(1, tot[1]), "rotation": acc[5] / max(1, tot[5])}}
    b.close()
    if not args.no_precision_error:
        out["fp32_vs_fp64"] = precision_error(ws[:1024], local)
    return out


def precision_error(ws, local, eq=5, npass=12):
    """The FP32 path's error against the FP64 path, replica by replica, on
    the same replicas with the same seeds: per replica <E> and the mean rotor
    axis z component <cos theta> over npass passes after eq, in each
    precision; the difference over the combined standard error (the g of each
    series from its pooled autocorrelation).  In FP64 a batch replica is the
    single-system chain, so this is the FP32 path against the FP64 plain
    path."""
    import numpy as np
    import pimc_gb300 as G
    ser = {}
    for mixed in (False, True):
        b = G.Batch(ws, device=local, mixed=mixed)
        b.run_passes(eq, 91)
        e, cz = [], []
        for k in range(npass):
            b.run_passes(1, 91)
            est = b.estimators()
            e.append(est[:, 0] + est[:, 1] + est[:, 2])
            cz.append(est[:, 3])
        b.close()
        ser[mixed] = (np.array(e), np.array(cz))
    out = {"replicas": len(ws), "passes": npass, "after": eq}
    for name, k in (("E", 0), ("cos_theta", 1)):
        x64, x32 = ser[False][k], ser[True][k]
        g64, g32 = pooled_inefficiency(x64), pooled_inefficiency(x32)
        se = np.sqrt(g64 * x64.var(axis=0, ddof=1) / npass + g32 * x32.var(axis=0, ddof=1) / npass)
        d = x32.mean(axis=0) - x64.mean(axis=0)
        ok = se > 0
        z = d[ok] / se[ok]
        out[name] = {"frac_within_2se": round(float(np.mean(np.abs(z) <= 2.0)), 4),
                     "median_abs_z": round(float(np.median(np.abs(z))), 3),
                     "mean_abs_diff": round(float(np.mean(np.abs(d))), 5),
                     "mean_diff": round(float(np.mean(d)), 5), "mean_se": round(float(np.mean(se)), 5)}
    return out


def run_tables(local, cpu):
    """The propagator-table generators, end to end through the C ABI (host
    eigen-decomposition, device sums, copy to host, symmetric fill):
    asymrho.f's full 181 x 361 x 361 table for nmv_prop/a-run (T 0.37 K, 128
    slices, A B C 0.6666525 0.2306476 0.1769383 cm^-1, J <= 66) and linden.f
    tables of 1500 points for the 4096 (T, Q) pairs of the replica batch.
    The CPU figures are the oracle's restatements of the reference's loops
    timed on a few points or tables and scaled to the whole job."""
    import numpy as np
    import pimc_gb300 as G
    import workloads as W
    out = {}
    abc = (0.6666525, 0.2306476, 0.1769383)
    G.asymrho(0.37, 128, -1, 10, 10, abc, 66, device=local)          # warm-up (context, allocations)
    t0 = time.perf_counter()
    rho, erot, esq, info = G.asymrho(0.37, 128, -1, 0, 180, abc, 66, device=local)
    gpu_s = time.perf_counter() - t0
    del rho, erot, esq
    computed = 181 * sum((p if p <= 90 else (180 - p if p <= 180 else (p - 180 if p <= 270 else 360 - p))) + 1
                         for p in range(361))
    out["asymrho"] = {"config": "nmv_prop/a-run: T 0.37 K, 128 slices, iodevn -1, A B C 0.6666525 0.2306476 "
                                "0.1769383 cm^-1, maxj 66; 181 x 361 x 361 grid", "gpu_s": round(gpu_s, 3),
                      "computed_points": computed}
    ws = W.config2(n=4096, seed=2024)
    T = np.array([w.temperature for w in ws])
    Q = np.array([w.nrotslices for w in ws])
    G.linden(T[:4], Q[:4], 0.39021, 1500, device=local)
    t0 = time.perf_counter()
    G.linden(T, Q, 0.39021, 1500, device=local)
    lin_s = time.perf_counter() - t0
    out["linden"] = {"config": "4096 tables x 1500 points, B 0.39021 cm^-1, (T, Q) of the replica batch",
                     "gpu_s": round(lin_s, 4)}
    if cpu:
        import oracle as O
        t0 = time.perf_counter()
        O.asymrho_points(0.37, 128, -1, abc, 66, [10, 10], [40, 200], [20, 30])
        per_pt = (time.perf_counter() - t0) / 2.0
        out["asymrho"]["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": "2 grid points (with the "
                                          "Wigner d list of one theta)", "s_per_point": round(per_pt, 4),
                                          "extrapolated_s": round(per_pt * computed, 1)}
        t0 = time.perf_counter()
        for i in range(16):
            O.linden(T[i], int(Q[i]), 0.39021, 1500)
        per_tab = (time.perf_counter() - t0) / 16
        out["linden"]["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": "16 tables",
                                         "s_per_table": round(per_tab, 5), "extrapolated_s": round(per_tab * 4096, 2)}
    return out


def run_worm(local, cpu, steps=5, warmup=2, replicas=32):
    """The worm branch of the pass loop (mc_main.cc:348-381) on config 0
    (CO2-like rotor + 8 He-4, P = 512, Q = 128) with WORM He4 1.0 16: per
    time slice the worm tries, the closed-path exchange bisection and
    centroid move, the rotor's bisection and rotational sweep.  One chain's
    passes (one CUDA graph per pass) timed with CUDA events on the library's
    stream; then `replicas` independent chains (own handles, streams and
    seeds) driven from host threads at once, timed by the wall clock between
    device synchronisations.  The CPU figure is the oracle's port of the same
    loop on a 64-slice sample, scaled to a pass."""
    import threading
    import torch
    import pimc_gb300 as G
    import workloads as W
    w = W.config0()
    w.worm = ("He4", 1.0, 16)
    s = G.Sampler(w, device=local)
    s.worm_init(0, 1.0, 16, w.density)
    s.worm_run(warmup, 32)              # the pass graph is built here, outside the timed region
    s.synchronize()
    ext = torch.cuda.ExternalStream(s.stream(), device=torch.device("cuda", local))
    l0 = s.launch_count()
    with torch.cuda.stream(ext):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.worm_run(steps, 32)
        e1.record(ext)
    s.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    tot, acc = s.worm_counters()
    out = {"workload": "config0 + WORM He4 1.0 16: 1 CO2-like rotor + 8 He-4, P=512, Q=128",
           "gpu_ms_per_pass": round(ms, 3), "slices_per_s": round(w.nslices / (ms / 1e3), 1),
           "launches_per_pass": int((s.launch_count() - l0) / steps),
           "worm_accept": {"open": acc[0] / max(1, tot[0]), "close": acc[1] / max(1, tot[1]),
                           "advance": acc[4] / max(1, tot[4]), "recede": acc[5] / max(1, tot[5]),
                           "swap": acc[6] / max(1, tot[6])}}
    s.close()
    if replicas > 1:
        ss = []
        for r in range(replicas):
            wr = W.config0(seed=1234 + 101 * r)
            sr = G.Sampler(wr, device=local)
            sr.worm_init(0, 1.0, 16, wr.density)
            ss.append(sr)

        def drive(n):
            errs = []

            def one(sr, seed):
                try:
                    sr.worm_run(n, seed)
                except Exception as e:          # re-raised on the main thread
                    errs.append(e)
            th = [threading.Thread(target=one, args=(sr, 500 + r)) for r, sr in enumerate(ss)]
            for t in th:
                t.start()
            for t in th:
                t.join()
            if errs:
                raise errs[0]
            for sr in ss:
                sr.synchronize()
            torch.cuda.synchronize()
        drive(warmup)
        t0 = time.perf_counter()
        drive(steps)
        el = time.perf_counter() - t0
        out["replicas"] = {"chains": replicas, "passes_each": steps, "wall_s": round(el, 3),
                           "slices_per_s": round(replicas * steps * w.nslices / el, 1),
                           "ms_per_pass_equivalent": round(el / (replicas * steps) * 1e3, 3),
                           "timing": "wall clock between device synchronisations, host threads one per chain"}
        for sr in ss:
            sr.close()
    if cpu:
        import oracle as O
        o = O.Oracle(w)
        o.worm_init(0, 1.0, 16, w.density)
        nth = os.cpu_count() or 1
        o.worm_run(0, 8, 5, nth)
        t0 = time.perf_counter()
        o.worm_run(8, 64, 6, nth)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"kind": "port", "cores": nth, "sample": "64 time slices of the worm pass loop",
                               "ms_per_pass": round(cs * w.nslices / 64 * 1e3, 1),
                               "slices_per_s": round(64 / cs, 1)}
        if replicas > 1:
            # the CPU's own best use of its cores for many chains: one
            # single-threaded chain per core, all at once
            os_ = []
            for r in range(nth):
                wr = W.config0(seed=1234 + 101 * r)
                orr = O.Oracle(wr)
                orr.worm_init(0, 1.0, 16, wr.density)
                orr.worm_run(0, 8, 5, 1)
                os_.append(orr)
            th = [threading.Thread(target=orr.worm_run, args=(8, 64, 6, 1)) for orr in os_]
            t0 = time.perf_counter()
            for t in th:
                t.start()
            for t in th:
                t.join()
            cs = time.perf_counter() - t0
            out["cpu_baseline"]["chains"] = {"chains": nth, "threads_each": 1,
                                             "sample": "64 time slices of each chain's worm pass loop",
                                             "slices_per_s": round(nth * 64 / cs, 1)}
    return out


# ------------------------------------------------------------ matched <E> SE

def pooled_inefficiency(E):
    """Statistical inefficiency g = 2 tau_int (in passes) of E[pass, replica]:
    each replica's series centred and scaled by its own variance, the
    normalised autocorrelation pooled over replicas, summed with Sokal's
    self-consistent window (the smallest W with W >= 5 tau(W))."""
    import numpy as np
    x = np.asarray(E, dtype=np.float64)
    x = x - x.mean(axis=0, keepdims=True)
    var = np.mean(x * x, axis=0)
    x = x[:, var > 0] / np.sqrt(var[var > 0])
    K = x.shape[0]
    tau = 0.5
    for k in range(1, K // 2):
        rho = float(np.mean(np.sum(x[:-k] * x[k:], axis=0) / (K - k)))
        tau += rho
        if k >= 5.0 * tau:
            break
    return max(2.0 * tau, 1e-3)


def series_stats(E):
    """Per-arm summary of an energy series E[pass, replica]: pooled g, the
    mean over replicas of the blocking SE of <E> (pimc_blocking_se) where the
    series is long enough, and the replica variances."""
    import numpy as np
    import pimc_gb300 as G
    E = np.asarray(E, dtype=np.float64)
    g = pooled_inefficiency(E)
    var = E.var(axis=0, ddof=1)
    se = None
    if E.shape[0] >= 16:
        se = float(np.mean([G.blocking_se(E[:, r])["se"] for r in range(E.shape[1])]))
    return {"g": round(g, 3), "passes": int(E.shape[0]), "mean_sd_K": round(float(np.mean(np.sqrt(var))), 4),
            "mean_blocking_se_K": None if se is None else round(se, 4)}, var


def batch_series(b, npasses, seed, eq, da=None):
    """eq untimed passes, then npasses passes each timed with CUDA events on
    the batch's stream; after each pass every replica's E = E_kin + E_pot +
    E_rot (pimc_batch_estimators, outside the events).  da: (mlp, escale) for
    delayed-acceptance passes (mlp None: the same passes without the
    screen)."""
    import numpy as np
    import torch
    ext = torch.cuda.ExternalStream(b.stream())
    run = (lambda n, sd: b.da_passes(n, sd, mlp=da[0], escale=da[1])) if da is not None else b.run_passes
    if eq:
        run(eq, seed)
    b.synchronize()
    E, ms = [], 0.0
    for k in range(npasses):
        with torch.cuda.stream(ext):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            run(1, seed)
            e1.record(ext)
        b.synchronize()
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
        est = b.estimators()
        E.append(est[:, 0] + est[:, 1] + est[:, 2])
    return np.array(E), ms / npasses


def work_units(w):
    """A replica's work per pass for scaling sampled pass times: its
    bead-moves, each weighted by the partners a move sums over."""
    return w.bead_moves_per_pass() * max(1, w.natoms - 1)


def scaled_total(ws, idx, ts):
    """The plain path's time for all replicas from the timed sample: the
    ratio estimator sum_r units_r * (sum_s t_s / sum_s units_s), and its
    standard error from the sample's scatter about that ratio."""
    import numpy as np
    u = np.array([work_units(ws[i]) for i in idx], dtype=np.float64)
    t = np.asarray(ts, dtype=np.float64)
    total_u = float(sum(work_units(w) for w in ws))
    ratio = t.sum() / u.sum()
    resid = t - ratio * u
    n = len(t)
    se = None
    if n > 1:
        se = total_u * float(np.sqrt(np.sum(resid ** 2) / (n - 1) / n)) / float(u.mean())
    return total_u * ratio, se


def single_pass_ms(ws, idx, seed, mixed=False):
    """One production pass of each chosen system on its own handle (the plain
    GPU path), CUDA events on the handle's stream after one untimed pass."""
    import torch
    import pimc_gb300 as G
    out = []
    for r in idx:
        s = G.Sampler(ws[r], mixed=mixed)
        s.run_passes(1, seed)
        s.synchronize()
        ext = torch.cuda.ExternalStream(s.stream())
        with torch.cuda.stream(ext):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            s.run_passes(1, seed)
            e1.record(ext)
        s.synchronize()
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
        s.close()
    return out


def matched(plain_pass_ms, plain_g, arms, c=0.05):
    """Time for every replica's <E> to reach a standard error of c times its
    own E fluctuation sd(E).  Every arm samples the same distribution (the
    exactness tests), so sd(E) is common to them and an arm needs
    n = g / c^2 passes, g its statistical inefficiency; the plain path runs
    the replicas one after another (its pass time is the sum over replicas),
    a batch runs them together.  var_ratio (each arm's replica variances over
    the mean of all arms') is reported as a check, not used."""
    import numpy as np
    n_plain = plain_g / (c * c)
    t_plain = n_plain * plain_pass_ms / 1e3
    out = {"target": "SE(<E>) = %.2f sd(E) per replica" % c,
           "plain": {"passes": round(n_plain, 1), "seconds": round(t_plain, 2)}}
    vbar = np.mean([np.sum(a["var"]) for a in arms.values()])
    for name, a in arms.items():
        n = a["g"] / (c * c)
        t = n * a["pass_ms"] / 1e3
        out[name] = {"passes": round(n, 1), "seconds": round(t, 3),
                     "var_ratio": round(float(np.sum(a["var"]) / vbar), 4), "vs_plain": round(t_plain / t, 2)}
    return out


def cpu_rate(ws, seconds, nthreads):
    """Bead-moves/s of the oracle port of the reference schedule (its timing
    build) over the systems ws in turn, each for an equal share of `seconds`
    (time slices 0, 1, ... of one pass, centroid moves at slice 0)."""
    import oracle as O
    bm, el = 0.0, 0.0
    for w in ws:
        o = O.Oracle(w, timing=True)
        t0 = time.perf_counter()
        done = 0
        while True:
            st, b = o.run_steps(done, 4, seed=99, nthreads=nthreads)
            if st != 0:
                raise RuntimeError("oracle run_steps failed: %d" % st)
            bm += b
            done += 4
            if time.perf_counter() - t0 >= seconds / len(ws) or done >= w.nslices:
                break
        el += time.perf_counter() - t0
    return bm / el


def gpu_pass_rate(w, local, mixed, passes=3):
    """Bead-moves/s of the single-system sampler on w: one untimed pass, then
    `passes` passes timed with CUDA events on the handle's stream."""
    import torch
    import pimc_gb300 as G
    s = G.Sampler(w, device=local, mixed=mixed)
    s.run_passes(1, 3)
    s.synchronize()
    ext = torch.cuda.ExternalStream(s.stream())
    with torch.cuda.stream(ext):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.run_passes(passes, 4)
        e1.record(ext)
    s.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / passes
    s.close()
    return w.bead_moves_per_pass() / (ms / 1e3)


def run_config_table(local, cpu_seconds=6.0):
    """Per configuration: the CPU oracle port of the reference schedule on all
    host cores and on one, the single-system GPU sampler in FP64 and on the
    FP32 path, and for the replica families the batch (FP32 path).  Replica
    families: the CPU and plain-GPU rates on a seeded sample of 8 replicas,
    the batch on all of them."""
    import numpy as np
    import pimc_gb300 as G
    import workloads as W
    ncores = os.cpu_count() or 1
    rng = np.random.default_rng(17)
    out = {}
    singles = {"config0": W.config0(), "config1": W.config1(), "config3": W.config3()}
    for name, w in singles.items():
        out[name] = {"cpu_all_cores": round(cpu_rate([w], cpu_seconds, ncores), 1),
                     "cpu_one_core": round(cpu_rate([w], cpu_seconds / 2, 1), 1),
                     "gpu_fp64": round(gpu_pass_rate(w, local, False), 1),
                     "gpu_fp32": round(gpu_pass_rate(w, local, True), 1)}
    for name, ws, shape, mode in (("config2", W.config2(), None, 0), ("config4", W.config4(), (8, 4), 1)):
        idx = rng.choice(len(ws), size=8, replace=False)
        sample = [ws[i] for i in idx]
        bm_s = sum(w.bead_moves_per_pass() for w in sample)
        t64 = sum(w.bead_moves_per_pass() / gpu_pass_rate(w, local, False, passes=1) for w in sample)
        t32 = sum(w.bead_moves_per_pass() / gpu_pass_rate(w, local, True, passes=1) for w in sample)
        b = G.Batch(ws, device=local, mixed=True)
        if shape:
            b.set_shape(*shape)
        if mode:
            b.set_rotation_mode(mode)
        _, ms = batch_series(b, 2, 23, 1)
        bm = b.bead_moves_per_pass()
        b.close()
        out[name] = {"cpu_all_cores": round(cpu_rate(sample, cpu_seconds, ncores), 1),
                     "cpu_one_core": round(cpu_rate(sample, cpu_seconds / 2, 1), 1),
                     "gpu_fp64": round(bm_s / t64, 1), "gpu_fp32": round(bm_s / t32, 1),
                     "gpu_batched_fp32": round(bm / (ms / 1e3), 1), "replicas": len(ws),
                     "sampled_replicas": [int(i) for i in idx]}
    out["cores"] = ncores
    out["host_cpu"] = host_cpu()
    return out


def run_fp64_pipe(local, iters=20000):
    """The FP64 pipe's occupancy rule (pimc_fp64_probe): warp-level FP64 FMA
    instructions retired per SM per microsecond, for one CTA per SM of 1-16
    warps with 1, 4 or 32 active lanes."""
    import pimc_gb300 as G
    rows = []
    for warps in (1, 2, 4, 8, 16):
        for lanes in (1, 4, 32):
            ms = G.fp64_probe(warps, lanes, iters, device=local)
            rows.append({"warps": warps, "lanes": lanes, "ms": round(ms, 4),
                         "warp_fma_per_sm_per_us": round(warps * iters * 8 / (ms * 1e3), 3)})
    return {"rows": rows}


def run_water_chains(local, steps, n=64):
    """A small case of the config-4 batch (the first n water-chain replicas'
    worth of the family, FP32 path, rotation mode 1, shape 8 x 4): one
    untimed pass, then `steps` passes timed with CUDA events (for profiling
    the half-sweep kernel on a small case)."""
    import pimc_gb300 as G
    import workloads as W
    ws = W.config4(n=n)
    b = G.Batch(ws, device=local, mixed=True)
    b.set_shape(8, 4)
    b.set_rotation_mode(1)
    _, ms = batch_series(b, steps, 3, 1)
    bm = b.bead_moves_per_pass()
    b.close()
    return {"workload": "config4 family, %d replicas, FP32 path, rotation mode 1" % n, "pass_ms": round(ms, 2),
            "bead_moves_per_s": round(bm / (ms / 1e3), 1)}


def crossover(w, line):
    """What a surrogate row must cost to pay in a delayed-acceptance screen
    of the rotor-solvent terms: the time of one exact rotor-pH2 term as the
    rotational kernels deliver it (the pass's rotation time over the
    reference's 2 R (N - 1) terms per slice move), FP64 and FP32 path,
    against the time of one surrogate row of the tensor-core forward kernel."""
    P, Q = w.nslices, w.nrotslices
    R = P // Q
    nr = sum(t["numb"] for t in w.types if t["molecule"] != 0)
    terms = P * Q * nr * 2 * R * (w.natoms - 1)
    main_ms = line["roofline"]["pass_ms_by_kind"]["rotation"]
    comp_ms = line["companion"]["pass_ms_by_kind"]["rotation"]
    f64, f32 = (main_ms, comp_ms) if line["config"]["precision"] == "fp64" else (comp_ms, main_ms)
    sr = line["surrogate"]["roofline"]
    row_ns = sr["ms_per_launch"] * 1e6 / line["surrogate"]["mlp_inference"]["rows"]
    t64, t32 = f64 * 1e6 / terms, f32 * 1e6 / terms
    return {"exact_term_ns_fp64": round(t64, 5), "exact_term_ns_fp32": round(t32, 5),
            "surrogate_row_ns": round(row_ns, 5), "row_over_fp64_term": round(row_ns / t64, 3),
            "row_over_fp32_term": round(row_ns / t32, 3),
            "what": "a screen spares exact terms only if a surrogate row costs less than the terms it replaces"}


def run_matched_se(local, mode="default", c4_replicas=512, c3_replicas=512, c4_shape=(8, 4)):
    """The metric itself: bead-moves/s at matched <E> standard error.

    Water chains (config 4): c4_replicas replicas of 1-8 water tops on a
    3 A chain + 0-32 pH2, T 0.5-2.0 K, P 512-2048, Q = P/4.  Arms: the plain
    GPU path -- each replica alone on the single-system sampler in FP64, the
    reference's arithmetic; its pass time measured on a seeded sample of
    replicas and scaled to all -- and the batch on the FP32 path with one
    launch per half-sweep over all replicas (rotation mode 1).  g (2 tau_int
    of E, in passes) comes from the batch's series; the plain chains make the
    same moves in FP64 (the statistics tests compare both precisions with the
    oracle), so their g is taken as the batch's.  The FP64 batch is timed on
    a replica subset, for its rate only.

    Water dimers (config 3 molecules, T 0.74 K, P = 512, Q = 256, levels 4,
    reduced slices so that a series fits the run): the plain GPU path, the
    batch with its rotational sweeps made by the delayed-acceptance kernels
    without a screen (plain Metropolis, in FP64 -- its g is the plain
    path's -- and on the FP32 path) and, on the FP32 path, with the screen of
    the surrogate trained on the plain sampler's own rows; in the "full" mode
    also the screened batch in FP64 and the batch with its sweeps in the
    half-sweep kernel.

    mode: "quick" (short series, for tests of the harness), "default" (the
    bench line), "full" (more sampled plain replicas, the extra dimer arm)."""
    import numpy as np
    import pimc_gb300 as G
    import workloads as W
    quick, full = mode == "quick", mode == "full"
    out = {"mode": mode}
    secs = {}
    t0 = time.perf_counter()

    def lap(name):
        nonlocal t0
        t1 = time.perf_counter()
        secs[name] = round(t1 - t0, 1)
        t0 = t1
    # ---------------- config 4
    ws = W.config4(n=c4_replicas)
    lap("config4_workloads")
    bm = sum(w.bead_moves_per_pass() for w in ws)
    rng = np.random.default_rng(11)
    k = 8 if quick else (40 if full else 24)
    idx = rng.choice(len(ws), size=min(k, len(ws)), replace=False)
    ts = np.array(single_pass_ms(ws, idx, 5))
    plain_ms, plain_ms_se = scaled_total(ws, idx, ts)
    lap("config4_plain")
    b = G.Batch(ws, mixed=True)
    b.set_shape(*c4_shape)
    rot_mode = 1
    b.set_rotation_mode(rot_mode)
    lap("config4_batch_setup")
    E, ms = batch_series(b, 4 if quick else 8, 21, 1)
    tot, acc = b.counters()
    b.close()
    lap("config4_batch_series")
    st, var = series_stats(E)
    arms = {"batched_fp32": dict(g=st["g"], var=var, pass_ms=ms, stats=st)}
    sub = [ws[i] for i in rng.choice(len(ws), size=min(64 if full else 16, len(ws)), replace=False)]
    b = G.Batch(sub, mixed=False)
    b.set_shape(*c4_shape)
    b.set_rotation_mode(rot_mode)
    _, ms64 = batch_series(b, 1, 22, 1)
    b.close()
    lap("config4_fp64_subset")
    bm_sub = sum(w.bead_moves_per_pass() for w in sub)
    out["config4"] = {
        "workload": "config4: %d replicas of 1-8 water tops (caleng) on a 3 A chain + 0-32 pH2 (vcord), "
                    "T 0.5-2.0 K, P 512-2048, Q=P/4, ROTDENSI 1" % len(ws),
        "bead_moves_per_pass": bm,
        "plain": {"bead_moves_per_s": round(bm / (plain_ms / 1e3), 1), "pass_ms_all_replicas": round(plain_ms, 1),
                  "pass_ms_se": None if plain_ms_se is None else round(plain_ms_se, 1),
                  "timed_replicas": int(len(idx)), "precision": "fp64", "g": st["g"],
                  "scaling": "ratio estimator on bead-moves x partners per replica"},
        "arms": {n: {"bead_moves_per_s": round(bm / (a["pass_ms"] / 1e3), 1), "pass_ms": round(a["pass_ms"], 2),
                     "precision": "fp32 tables, pair terms and densities, fp64 sums and accepts", **a["stats"]}
                 for n, a in arms.items()},
        "accept_ratios": {"pH2 bisection": acc[1] / max(1, tot[1]), "water bisection": acc[4] / max(1, tot[4]),
                          "rotation": acc[5] / max(1, tot[5])},
        "batched_fp64_subset": {"replicas": len(sub), "pass_ms": round(ms64, 1),
                                "bead_moves_per_s": round(bm_sub / (ms64 / 1e3), 1)},
        "shape": {"warps_per_cta": c4_shape[0], "ctas_per_sm_bound": c4_shape[1], "rotation_mode": rot_mode},
        "time_to_se": matched(plain_ms, st["g"], arms)}
    # ---------------- water dimers with the surrogate
    d0 = W.config3(seed=300, nslices=512, nrotslices=256, levels=4)
    dims = [d0] + [W.config3(seed=300 + r, nslices=512, nrotslices=256, levels=4, tables=d0.tables)
                   for r in range(1, c3_replicas)]
    bmd = sum(w.bead_moves_per_pass() for w in dims)
    lap("dimer_workloads")
    ts = np.array(single_pass_ms(dims, range(min(4, len(dims))), 7))
    plain_d_ms = float(ts.mean()) * len(dims)           # identical systems: the mean pass time
    # training rows from the plain sampler (dimer features, exact caleng energies)
    s = G.Sampler(dims[0])
    s.run_passes(2, 3)
    xs, es = [], []
    for kk in range(16 if quick else 64):
        s.da_sweeps(4, 100 + kk)
        f, e = s.da_samples()
        xs.append(f)
        es.append(e)
    s.close()
    x, e = np.concatenate(xs), np.concatenate(es)
    mu, sd = float(e.mean()), float(e.std())
    m = G.Mlp(device=local)
    r0 = np.random.default_rng(5)
    m.set_weights(r0.normal(0, 1 / np.sqrt(6), (6, 256)), np.zeros(256), r0.normal(0, 1 / 16, (256, 256)),
                  np.zeros(256), r0.normal(0, 1 / 16, (256, 256)), np.zeros(256), r0.normal(0, 1 / 16, 256), 0.0)
    m.train(x, (e - mu) / sd, epochs=4 if quick else 12, batch=8192, lr=2e-3, seed=6)
    lap("dimer_plain_and_training")
    darms = {}
    npd = 6 if quick else 32
    eq = 1 if quick else 4
    # the unscreened and the screened batch (FP32 path); the unscreened one in
    # FP64 too (the plain path's arithmetic, its g is the plain path's)
    runs = [("batched_da_exact", (None, sd), False), ("batched_da_exact_fp32", (None, sd), True),
            ("batched_surrogate_fp32", (m, sd), True)]
    if full:
        runs += [("batched_surrogate", (m, sd), False), ("batched_plain", None, False)]
    for name, da, mixed in runs:
        b = G.Batch(dims, mixed=mixed)
        if da is None:
            b.set_rotation_mode(1)
        E, ms = batch_series(b, npd, 31, eq, da=da)
        st, var = series_stats(E)
        tot, acc = b.counters()
        darms[name] = dict(g=st["g"], var=var, pass_ms=ms, stats=st, accept_rot=float(acc[2] / max(1, tot[2])))
        b.close()
        lap("dimer_" + name)
    m.close()
    out["section_seconds"] = secs
    g_plain = darms["batched_da_exact"]["g"]
    out["config3_dimers"] = {
        "workload": "config3 molecules: %d water dimers (caleng), T=0.74 K, P=512, Q=256, levels 4 (slices "
                    "reduced from 4096/2048 so that a series fits the run)" % len(dims),
        "bead_moves_per_pass": bmd,
        "plain": {"bead_moves_per_s": round(bmd / (plain_d_ms / 1e3), 1), "pass_ms_all_replicas": round(plain_d_ms, 1),
                  "timed_replicas": int(len(ts)), "precision": "fp64", "g": g_plain,
                  "g_source": "the unscreened batch arm (the same Metropolis moves)"},
        "arms": {n: {"bead_moves_per_s": round(bmd / (a["pass_ms"] / 1e3), 1), "pass_ms": round(a["pass_ms"], 2),
                     "accept_rot": round(a["accept_rot"], 4), **a["stats"]} for n, a in darms.items()},
        "surrogate": {"training_rows": int(len(x)), "energy_sd_K": round(sd, 2)},
        "time_to_se": matched(plain_d_ms, g_plain, darms)}
    return out


def run_surrogate(local, quick=False, replicas=32):
    """The surrogate with delayed acceptance on config 3 (2 water-like tops, caleng, T 0.74 K,
    P = 4096, Q = 2048): training data emitted by the plain sampler (dimer
    features and exact caleng energies of every translational slice), the
    surrogate MLP trained on the GPU by its tcgen05 kernels, then plain and
    delayed-acceptance rotational sweeps timed with CUDA events.  Also the
    surrogate's inference rate on a large batch against the tensor-core
    peak.  Then `replicas` independent dimer systems (own handles, streams
    and seeds, one trained surrogate shared read-only) make plain and
    delayed-acceptance sweeps at once from one host thread each, timed by
    the wall clock between device synchronisations."""
    import threading
    import numpy as np
    import torch
    import pimc_gb300 as G
    import workloads as W
    w = W.config3()
    s = G.Sampler(w, device=local)
    ext = torch.cuda.ExternalStream(s.stream(), device=torch.device("cuda", local))
    s.da_sweeps(20, 11)
    ncall = 64 if quick else 256
    t0 = time.perf_counter()
    xs, es = [], []
    for k in range(ncall):
        s.da_sweeps(2, 100 + k)
        f, e = s.da_samples()
        xs.append(f)
        es.append(e)
    t_collect = time.perf_counter() - t0
    x, e = np.concatenate(xs), np.concatenate(es)
    mu, sd = float(e.mean()), float(e.std())
    nho = 16384
    m = G.Mlp(device=local)
    rng = np.random.default_rng(5)
    m.set_weights(rng.normal(0, 1 / np.sqrt(6), (6, 256)), np.zeros(256), rng.normal(0, 1 / 16, (256, 256)),
                  np.zeros(256), rng.normal(0, 1 / 16, (256, 256)), np.zeros(256), rng.normal(0, 1 / 16, 256), 0.0)
    epochs = 12
    t0 = time.perf_counter()
    losses = m.train(x[:-nho], (e[:-nho] - mu) / sd, epochs=epochs, batch=8192, lr=2e-3, seed=6)
    t_train = time.perf_counter() - t0
    pred = m.forward(x[-nho:]) * sd + mu
    rms = float(np.sqrt(np.mean((pred - e[-nho:]) ** 2)))

    def timed(nsw, mlp):
        with torch.cuda.stream(ext):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            st = s.da_sweeps(nsw, 999, mlp=mlp, escale=sd)
            b.record(ext)
        s.synchronize()
        torch.cuda.synchronize()
        return a.elapsed_time(b), st

    nsw = 20 if quick else 100
    # warm-up calls of the same shape: a call is captured as a CUDA graph once
    timed(nsw, None)
    ms_plain, st_plain = timed(nsw, None)
    timed(nsw, m)
    ms_da, st_da = timed(nsw, m)
    # inference rate of the tensor-core layers on one large batch
    xb = np.tile(x[:8192], (64, 1))
    m.forward(xb[:8192])
    t0 = time.perf_counter()
    m.forward(xb)
    t_inf = time.perf_counter() - t0
    flop_row = 2 * 2 * 256 * 256
    # the forward kernel alone, rows resident in HBM, CUDA events on its stream
    mext = torch.cuda.ExternalStream(m.stream(), device=torch.device("cuda", local))
    reps = 10
    with torch.cuda.stream(mext):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        m.forward_resident(len(xb))
        a.record(mext)
        for _ in range(reps):
            m.forward_resident(len(xb))
        b.record(mext)
    torch.cuda.synchronize()
    k_ms = a.elapsed_time(b) / reps
    peak_tf, peak_kind = bf16_peak()
    k_tf = len(xb) * flop_row / (k_ms / 1e3) / 1e12
    out = {"workload": "config3: 2 water-like tops (A,B,C = 27.9, 14.5, 9.3 cm^-1), caleng, T=0.74 K, P=4096, Q=2048",
           "training": {"samples": int(len(x) - nho), "collect_s": round(t_collect, 2), "epochs": epochs,
                        "train_s": round(t_train, 2), "loss_first_last": [round(float(losses[0]), 4),
                                                                          round(float(losses[-1]), 4)],
                        "heldout_rms_K": round(rms, 2), "energy_std_K": round(sd, 2)},
           "plain": {"moves_per_s": round(st_plain[0] / (ms_plain / 1e3), 1),
                     "accept": round(st_plain[2] / st_plain[0], 4)},
           "delayed_acceptance": {"moves_per_s": round(st_da[0] / (ms_da / 1e3), 1),
                                  "stage1_pass": round(st_da[1] / st_da[0], 4),
                                  "accept": round(st_da[2] / st_da[0], 4),
                                  "exact_evals_per_move": round(st_da[3] / st_da[0], 4)},
           "mlp_inference": {"rows": int(len(xb)), "s_end_to_end": round(t_inf, 4),
                             "tensor_tflops_end_to_end": round(len(xb) * flop_row / t_inf / 1e12, 2)},
           "roofline": {"bound": "tensor", "kernel": "k_mlp_forward (tcgen05 layers 2-3)",
                        "achieved": round(k_tf, 2), "peak": peak_tf, "unit": "TFLOP/s",
                        "frac": round(k_tf / peak_tf, 5), "ms_per_launch": round(k_ms, 4),
                        "flop_per_row": flop_row, "peak_source": peak_kind}}
    if replicas > 1:
        hs = [s] + [G.Sampler(W.config3(seed=77 + 13 * r), device=local) for r in range(1, replicas)]

        def drive(nsw, mlp):
            res, errs = [None] * len(hs), []

            def one(r):
                try:
                    res[r] = hs[r].da_sweeps(nsw, 3000 + r, mlp=mlp, escale=sd)
                except Exception as ex:          # re-raised on the main thread
                    errs.append(ex)
            th = [threading.Thread(target=one, args=(r,)) for r in range(len(hs))]
            t0 = time.perf_counter()
            for t in th:
                t.start()
            for t in th:
                t.join()
            for h in hs:
                h.synchronize()
            torch.cuda.synchronize()
            el = time.perf_counter() - t0
            if errs:
                raise errs[0]
            moves = sum(float(r[0]) for r in res)
            return {"moves_per_s": round(moves / el, 1), "wall_s": round(el, 3),
                    "accept": round(sum(float(r[2]) for r in res) / moves, 4),
                    "exact_evals_per_move": round(sum(float(r[3]) for r in res) / moves, 4)}
        nb = 20 if quick else 200
        drive(nb, None)                 # warm-up of the same shape (graph capture)
        bp = drive(nb, None)
        drive(nb, m)
        bd = drive(nb, m)
        out["batched"] = {"systems": replicas, "sweeps_each": nb, "plain": bp, "delayed_acceptance": bd,
                          "timing": "wall clock between device synchronisations, host threads one per system",
                          "vs_single_plain": round(bd["moves_per_s"] / out["plain"]["moves_per_s"], 2)}
        for h in hs[1:]:
            h.close()
    m.close()
    s.close()
    return out


def main():
    args = parse()
    rank, local, world = dist_env()
    dist = dist_init(world)
    ncores = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return 0
        w = workload(0)
        rate, sample = cpu_baseline(w, args.cpu_seconds, ncores)
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "host_cpu": host_cpu()},
                "cpu_baseline": {"value": rate, "unit": UNIT, "cores": ncores, "kind": "port", "sample": sample},
                "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    if args.only is not None:
        if rank == 0:
            run = {"tables": lambda: run_tables(local, not args.no_cpu),
                   "worm": lambda: run_worm(local, not args.no_cpu, steps=args.steps, warmup=args.warmup,
                                            replicas=args.worm_replicas),
                   "surrogate": lambda: run_surrogate(local, replicas=args.da_replicas),
                   "matched_se": lambda: run_matched_se(local, mode=args.se_mode),
                   "water_chains": lambda: run_water_chains(local, args.steps),
                   "config_table": lambda: run_config_table(local),
                   "fp64_pipe": lambda: run_fp64_pipe(local)}[args.only]
            print(json.dumps({"part": args.only, **run()}), flush=True)
        return 0
    line, w = run_gb300(args, rank, local, world, dist)
    if rank == 0:
        if not args.no_cpu:
            rate, sample = cpu_baseline(w, args.cpu_seconds, ncores)
            rate1, sample1 = cpu_baseline(w, args.cpu_seconds / 2, 1)
            line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": ncores, "kind": "port", "sample": sample,
                                    "host_cpu": host_cpu(),
                                    "one_thread": {"value": rate1, "cores": 1, "sample": sample1}}
        if not args.no_tables and world == 1:
            line["tables"] = run_tables(local, not args.no_cpu)
        if not args.no_worm and world == 1:
            line["worm"] = run_worm(local, not args.no_cpu, replicas=args.worm_replicas)
        if not args.no_surrogate and world == 1:
            line["surrogate"] = run_surrogate(local, replicas=args.da_replicas)
        if not args.no_matched_se and world == 1:
            line["matched_se"] = run_matched_se(local, mode=args.se_mode)
        if "surrogate" in line and "companion" in line:
            line["surrogate_crossover"] = crossover(w, line)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
