#!/usr/bin/env python
"""Benchmark of the collision-query hot path on one or more GPUs.

Default workload (N=1): batched first-contact queries on the interlocking-tori
meshes -- 1M segments per GPU, start states uniform in [-2, 2]^3 (world units)
with Shoemake rotations, ends displaced by N(0, 0.3^2) and rotated by
U[0, pi], stepped at verify_delta = 0.001 in the unit frame exactly as
UnitWorld::transitStateToWithContact does.  The metric is collision checks per
second: the isValid calls the sequential reference loop makes for the batch
(first contact + 1 per colliding segment, every step of a free one).

One "step" = one pw_segments_first_contact call over the whole resident batch.
Launch: python bench.py [--gpus N --steps K --warmup W] [--impl reference];
N > 1 runs under torch.distributed.run, one rank per GPU, weak scaling (each
rank its own seeded batch, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from puzzletunneldiscovery_gb300 import workloads as W  # noqa: E402

UNIT = "checks/s"
DELTA = 0.001
# per-unit algorithmic bytes of the traversal kernel: each node-pair test reads two
# FP32 boxes, each leaf test two FP32 triangles, each segment its two states and
# writes its first-contact step
BYTES_NODE_PAIR = 2 * 32      # env node + robot node (two float4 each: aligned boxes)
BYTES_NODE_PAIR_OBB = 2 * 80  # oriented boxes: centre, half-extents and three axis rows (five float4)
BYTES_LEAF_PAIR = 2 * 48      # env triangle + robot triangle (three float4 each)
BYTES_SEGMENT = 2 * 56 + 4    # two states in, one int32 out


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


WORKLOADS = {
    # name: (metric, meshes, default units per GPU)
    "segments": ("collision checks/sec (first-contact segment queries, interlocking tori)",
                 W.cfg_interlocking_tori, 1_000_000),
    "plate": ("collision checks/sec (is_valid_state, perforated plate vs torus knot)", W.cfg_plate_knot, 20_000_000),
    "surrogate": ("verified collision-free samples/sec (surrogate-guided, interlocking tori)",
                  W.cfg_interlocking_tori, 200_000_000),
    "narrow": ("escapes through a plate hole/sec (surrogate-guided narrow-passage search, plate vs torus knot)",
               W.cfg_plate_knot, 4_000_000),
    "ompl": ("motions checked/sec (OMPL discrete motion check, validate_motion_pairs, alpha puzzle)",
             lambda: _alpha_ompl()[0], 1_000_000),
    # the other rows of the path, each on the interlocking tori
    "disentangled": ("is_disentangled checks/sec (interlocking tori)", W.cfg_interlocking_tori, 20_000_000),
    "contacts": ("contact enumerations/sec (intersecting_segments on colliding interlocking-tori states)",
                 W.cfg_interlocking_tori, 65536),
    "keyconf": ("key-configuration candidates checked/sec (enum_free_configuration, 256 spins, only_median)",
                W.cfg_interlocking_tori, 8192),
    "visibility": ("is_valid_transition pairs/sec (calculate_visibility_matrix of free interlocking-tori "
                   "states, verify_magnitude 0.00625)", W.cfg_interlocking_tori, 2048),
    "touch": ("touch samples/sec (calc_touch: 128 random segments per key to first contact)",
              W.cfg_interlocking_tori, 8192),
}
ROW_WORKLOADS = ("disentangled", "contacts", "keyconf", "touch", "visibility")
KEYCONF_SPINS = 256          # envconfig.py:134 NumberOfRotations
KEYCONF_MARGIN = 1e-6        # envconfig.py:136 Margin
TOUCH_PER_KEY = 128          # envconfig.py:141 OversamplingClearanceSample
VIS_DELTA = 0.0125 * 4 / 8   # visibility-finder.py:33, the visibility matrix's verify_magnitude
BVH_KIND = "topdown"         # the worlds' BVH hierarchy (--bvh)
# OMPL motion workload: collision resolution and the spread of the motions' targets (OMPL units)
OMPL_CDRES = 0.01
OMPL_SIGMA = 2.0
# proposal network: FLOPs per scored state (9 -> 256 x4 -> 1; the padded input columns are not counted)
MLP_FLOP_PER_ROW = 2 * (9 * 256 + 3 * 256 * 256 + 256)


def _quat_matrix(q):
    """Rotation matrix of a unit quaternion (w, x, y, z)."""
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _alpha_ompl():
    """The alpha puzzle (its meshes and solution path, tests/golden/alpha_puzzle.npz)
    with the path's states written in the OMPL frame of a world whose robot centre
    is enforced to the puzzle's centre c: t_ompl = t + R(q) (m - c), m the robot's
    float vertex mean, so that translateOMPLStateToUnitState gives back the
    path's unit-frame states.  Returns ((Ve, Fe, Vr, Fr), c, path in the OMPL frame)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "alpha_puzzle.npz"))
    c = g["center"].astype(np.float32)
    acc = np.zeros(3, dtype=np.float32)
    for v in g["Vr"].astype(np.float32):
        acc = acc + v
    d = (acc / np.float32(len(g["Vr"])) - c).astype(np.float64)
    P = g["path_wlast"].astype(np.float64).copy()
    for i, p in enumerate(P):
        q = np.array([p[6], p[3], p[4], p[5]])
        P[i, :3] = p[:3] + _quat_matrix(q / np.linalg.norm(q)) @ d
    return (g["Ve"], g["Fe"], g["Vr"], g["Fr"]), c, P


def _ompl_motions(P, n, seed):
    """n motions from a path state to another path state displaced by N(0, sigma^2)
    per axis, in the path's box widened by 20 on every side (the bounds of the
    state space)."""
    rng = np.random.default_rng(1000 + seed)
    i = rng.integers(0, len(P), n)
    j = rng.integers(0, len(P), n)
    B = P[j].copy()
    B[:, :3] += rng.normal(0.0, OMPL_SIGMA, (n, 3))
    return np.ascontiguousarray(P[i]), B, P[:, :3].min(axis=0) - 20.0, P[:, :3].max(axis=0) + 20.0


def _ompl_oracle():
    from oracle import oracle as O
    O.build()
    (Ve, Fe, Vr, Fr), c, P = _alpha_ompl()
    return O.OracleWorld(Ve, Fe, Vr, Fr, center=c), P


def _ompl_cpu(ow, A, B, lo, hi, target_s, start_n=2048):
    """The oracle's validateMotionPairs (OMPL's early-exit order, all host threads) on a
    sample of the motions grown until it takes about target_s: (motions/s, sample
    size, checks per motion, seconds, verdicts)."""
    cores = os.cpu_count() or 1
    n = min(start_n, len(A))
    while True:
        t0 = time.perf_counter()
        v, c = ow.ompl_check_motions(A[:n], B[:n], lo, hi, OMPL_CDRES, nthreads=cores)
        dt = time.perf_counter() - t0
        if dt >= target_s or n >= len(A):
            break
        n = min(len(A), max(n * 2, int(n * target_s / max(dt, 1e-3) * 1.1)))
    return n / dt, n, float(c.mean()), dt, v


def run_ompl(args):
    """--workload ompl: pw_ompl_check_motions over a resident batch of motions."""
    import torch
    import torch.distributed as dist

    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import ompl_compat as OC

    ws, rank, local = _dist_env()
    if ws > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    (Ve, Fe, Vr, Fr), c, P = _alpha_ompl()
    uw = pw.UnitWorld(local)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.enforceRobotCenter(c)
    uw.scaleToUnit()
    uw.set_bvh(BVH_KIND)
    uw.angleModel(0.0, 0.0)
    A, B, lo, hi = _ompl_motions(P, args.n, rank)
    a = torch.from_numpy(A).to(dev)
    b = torch.from_numpy(B).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # the BVH hierarchy and the states kernel's node boxes, picked on the motions themselves
    from puzzletunneldiscovery_gb300.autotune import pick_bvh
    picked = pick_bvh(uw, run=lambda: OC._check_motions_dev(uw, a, b, lo, hi, OMPL_CDRES)[0], kernel=0)
    box_kind, box_ms = picked["boxes"]["states"], picked["ms"]
    for _ in range(args.warmup):
        OC._check_motions_dev(uw, a, b, lo, hi, OMPL_CDRES)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    checked, launches = [], 0
    with ClockSampler(local) as clk:
        barrier()
        for i in range(args.steps):
            flush.zero_()                      # L2 flush between timed steps (not timed)
            ev[i][0].record(stream)
            v, n_states = OC._check_motions_dev(uw, a, b, lo, hi, OMPL_CDRES)
            ev[i][1].record(stream)
            checked.append(n_states)
            launches += uw.last_stats()["kernel_launches"]
        barrier()
    step_ms = [s0.elapsed_time(s1) for s0, s1 in ev]
    tot_ms, tot_motions = max_time_sum_units(sum(step_ms), args.n * args.steps, ws, dev)
    value = tot_motions / (tot_ms / 1e3)
    verdicts = v.cpu().numpy()

    # end to end through the public host-array call: motions copied in, verdicts out, every step
    ha = torch.from_numpy(A).pin_memory().numpy()
    hb = torch.from_numpy(B).pin_memory().numpy()
    e2e_ms = 0.0
    barrier()
    for i in range(args.steps):
        flush.zero_()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        hv, _ = OC.check_motions_discrete(uw, ha, hb, lo, hi, OMPL_CDRES)
        s1.record(stream)
        torch.cuda.synchronize(dev)
        e2e_ms += s0.elapsed_time(s1)
    if not np.array_equal(hv, verdicts.astype(np.int32)):
        raise RuntimeError("host-array path disagrees with the device path")
    e2e_ms, e2e_motions = max_time_sum_units(e2e_ms, args.n * args.steps, ws, dev)
    e2e_value = e2e_motions / (e2e_ms / 1e3)

    if rank != 0:
        if ws > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    states = checked[-1]
    ms = tot_ms / args.steps
    # per checked state: generated and written (56 B), read by the check (56 B), its verdict
    # written and read (2 B); per motion: both ends read by the count and state kernels
    # (4 x 56 B), its count and offset (16 B) and verdict (1 B)
    alg_bytes = states * 114 + args.n * (4 * 56 + 17)
    peak, peak_kind = _peaks()
    achieved = alg_bytes / (ms / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "whole call (k_ompl_counts, k_ompl_states, k_states, k_ompl_reduce)",
            "peak_source": peak_kind, "algorithmic_bytes": alg_bytes,
            "note": "the states pass is bound by the traversal's SM issue, as in the plate workload"}
    cpu, cpu_mism, cpu_n = None, None, 0
    if ws == 1 and not args.no_cpu_baseline:
        ow, _ = _ompl_oracle()
        cv, cn, cpm, cdt, ov = _ompl_cpu(ow, A, B, lo, hi, args.cpu_seconds)
        cpu_mism, cpu_n = int((ov != verdicts[:cn]).sum()), int(cn)
        if cpu_mism:
            raise RuntimeError("GPU verdicts differ from the oracle's on the CPU sample")
        cpu = {"value": cv, "unit": "motions/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "first %d motions of the batch (OMPL's early-exit order, %.2f states checked per "
                         "motion, %.1f s); verdicts equal the GPU's" % (cn, cpm, cdt)}
    line = {"metric": WORKLOADS["ompl"][0], "value": value, "unit": "motions/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 state math + f32 traversal",
            "data": "synthetic (seeded motions between the alpha puzzle's path states)",
            "config": {"workload": "validate_motion_pairs/alpha_puzzle", "n_motions_per_gpu": args.n,
                       "cdres": OMPL_CDRES, "target_sigma": OMPL_SIGMA,
                       "bounds": [lo.tolist(), hi.tolist()],
                       "l2": "flushed (256 MB write) between timed steps; per-step working set > L2",
                       "parallelism": "replicas" if ws == 1 else "shard-per-rank (weak)"},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "motions/s", "h2d_bytes_per_step": int(args.n * 112 * ws),
                    "d2h_bytes_per_step": int(args.n * ws)},
            "clocks": clk.summary(),
            # segment counts; per pass its counts, then per window of its states: generation,
            # traversal, re-test, reduction (the library's own count)
            "gpu_launches": launches,
            "detail": {"mismatches": cpu_mism, "mismatch_sample": cpu_n,
                       "node_boxes": {"states": box_kind, "ms": box_ms}, "bvh": picked["bvh"],
                       "states_checked_per_step": states, "states_per_motion": states / args.n,
                       "valid_fraction": float(verdicts.mean()), "step_ms": step_ms}}
    print(json.dumps(line))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def run_ompl_reference(args):
    """--impl reference --workload ompl: the oracle's validateMotionPairs on the host cores."""
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    ow, P = _ompl_oracle()
    A, B, lo, hi = _ompl_motions(P, args.n, 0)
    cores = os.cpu_count() or 1
    sample = 50 * args.ref_sample
    times = []
    for it in range(args.warmup + args.steps):
        s0 = (it * sample) % max(1, args.n - sample)
        t0 = time.perf_counter()
        ow.ompl_check_motions(A[s0:s0 + sample], B[s0:s0 + sample], lo, hi, OMPL_CDRES, nthreads=cores)
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = sample * len(times) / sum(times)
    line = {"impl": "reference", "metric": WORKLOADS["ompl"][0], "value": value, "unit": "motions/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, same motions as the GPU arm)",
            "config": {"workload": "validate_motion_pairs/alpha_puzzle", "n_motions_per_gpu": args.n,
                       "cdres": OMPL_CDRES, "sample_per_step": sample},
            "cpu_baseline": {"value": value, "unit": "motions/s", "cores": cores, "kind": "port",
                             "sample": "%d motions per step of the %d-motion batch" % (sample, args.n)},
            "e2e": {"value": value, "unit": "motions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _meshes(workload="segments"):
    return WORKLOADS[workload][1]()


def _batch(n, scale, seed, workload="segments", Ve=None):
    if workload == "plate":
        lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
        return W.uniform_states(n, lo, hi, scale, seed=seed), None
    return W.segment_batch(n, -2.0, 2.0, scale, seed=seed)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        # samples go to a temporary file (override with PW_BENCH_CLOCKS_DIR); the
        # JSON line carries their summary
        self.path = os.path.join(os.environ.get("PW_BENCH_CLOCKS_DIR", tempfile.gettempdir()),
                                 "bench_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return None
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 7 and parts[0].replace(".", "").isdigit():
                    rows.append(parts)
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[0]) for r in rows]
        mx = max(float(r[1]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


class Work:
    """One workload: its meshes, per-rank batch, GPU call and CPU-oracle call."""

    def __init__(self, name, n, seed, scale, Ve):
        self.name = name
        self.n = n
        self.metric = WORKLOADS[name][0]
        self.q0, self.q1 = _batch(n, scale, seed, name, Ve)

    def gpu(self, uw, a, b):
        if self.name == "plate":
            return uw.is_valid_states(a)
        return uw.first_contact_steps(a, b, DELTA)

    def gpu_host(self, uw, ha, hb):
        """The same call on host batches (the public host-array entry points: the
        copies of one chunk overlap the checks of the previous one)."""
        if self.name == "plate":
            return uw.is_valid_states_host(ha)
        return uw.first_contact_steps_host(ha, hb, DELTA)

    def cpu(self, ow, lo, hi, threads):
        """(reference checks, seconds, result) of the oracle on units lo..hi; the
        result is in the GPU call's encoding (first-contact steps, or 1 = free)."""
        t0 = time.perf_counter()
        if self.name == "plate":
            res = ow.is_valid(self.q0[lo:hi], nthreads=threads).astype(np.uint8)
            checks = hi - lo
        else:
            res, c = ow.segments_first_contact(self.q0[lo:hi], self.q1[lo:hi], DELTA, mode=0, nthreads=threads)
            checks = int(c.sum())
        return checks, time.perf_counter() - t0, res

    def bytes_in(self):
        return self.n * 56 * (1 if self.name == "plate" else 2)

    def bytes_out(self):
        return self.n * (1 if self.name == "plate" else 4)


def cpu_baseline(work, gpu_result, target_s=12.0):
    """The oracle (CPU restatement of the reference path) on a bounded sample of
    the timed batch, all host threads, and its results compared with the GPU's
    on that sample.  Returns (cpu_baseline dict, parity dict)."""
    from oracle import oracle as O
    O.build()
    Ve, Fe, Vr, Fr = _meshes(work.name)
    ow = O.OracleWorld(Ve, Fe, Vr, Fr)
    cores = os.cpu_count() or 1
    n = 128 if work.name == "segments" else 8192
    while True:
        n = min(n, work.n)
        checks, dt, res = work.cpu(ow, 0, n, cores)
        if dt >= target_s or n >= work.n:
            break
        n = min(work.n, max(n * 2, int(n * target_s / max(dt, 1e-3) * 1.1)))
    unit_name = "segments" if work.name == "segments" else "states"
    # the same oracle on one thread, on the sample's first part (about a quarter of target_s)
    n1 = max(1, min(n, int(n * (target_s / 4.0) / max(dt * cores, 1e-3))))
    checks1, dt1, res1 = work.cpu(ow, 0, n1, 1)
    g = np.asarray(gpu_result[:n])
    mism = int((g != res).sum()) + int((g[:n1] != res1).sum())
    what = ("first-contact step index (or -1) of every segment" if work.name == "segments"
            else "is_valid_state verdict of every state")
    parity = {"mismatches": mism, "mismatch_sample": int(n), "compared": what,
              "sample": "first %d %s of the timed batch (the CPU-baseline sample), against the timed steps' "
                        "results" % (n, unit_name)}
    cpu = {"value": float(checks) / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": "first %d %s of the rank-0 batch (%d reference checks, %.1f s)" % (n, unit_name, checks, dt),
           "single_thread": {"value": float(checks1) / max(dt1, 1e-9), "unit": UNIT, "cores": 1,
                             "sample": "first %d %s (%d reference checks, %.1f s)" % (n1, unit_name, checks1, dt1)}}
    return cpu, parity


def run_reference(args):
    """--impl reference: the CPU restatement of the reference path, timed on the host cores."""
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    Ve, Fe, Vr, Fr = _meshes(args.workload)
    ow = O.OracleWorld(Ve, Fe, Vr, Fr)
    cores = os.cpu_count() or 1
    work = Work(args.workload, args.n, 0, ow.scene_scale, Ve)
    sample = args.ref_sample if args.workload == "segments" else 100 * args.ref_sample
    times, checks = [], []
    for it in range(args.warmup + args.steps):
        lo = (it * sample) % max(1, work.n - sample)
        c, dt, _ = work.cpu(ow, lo, lo + sample, cores)
        if it >= args.warmup:
            times.append(dt)
            checks.append(c)
    value = sum(checks) / sum(times)
    line = {"impl": "reference", "metric": work.metric, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, same batch as the GPU arm)",
            "config": {"workload": args.workload, "units_per_gpu": args.n, "verify_delta": DELTA,
                       "sample_per_step": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d units per step of the %d-unit batch" % (sample, args.n)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def max_time_sum_units(ms, units, world, device):
    """Whole-job figures over the ranks: the slowest rank's time and the units all
    ranks processed (weak scaling: each rank times its own batch)."""
    if world <= 1:
        return float(ms), float(units)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(units)], device=device, dtype=torch.float64)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t.item()), float(c.item())


def run_ours(args):
    import torch
    import torch.distributed as dist

    import puzzletunneldiscovery_gb300 as pw

    ws, rank, local = _dist_env()
    if ws > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    Ve, Fe, Vr, Fr = _meshes(args.workload)
    uw = pw.UnitWorld(local)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.set_bvh(BVH_KIND)
    uw.angleModel(0.0, 0.0)
    work = Work(args.workload, args.n, rank, uw.scene_scale, Ve)
    a = torch.from_numpy(work.q0).to(dev)
    b = torch.from_numpy(work.q1).to(dev) if work.q1 is not None else None
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    tuned = None
    if not args.no_autotune:
        # launch configuration picked by the autotuner on a sample of this rank's own batch
        from puzzletunneldiscovery_gb300.autotune import tune_segments, tune_states
        if args.workload == "plate":
            r = tune_states(uw, a[: min(args.n, 2_000_000)], reps=1)
        else:
            m = min(args.n, 100_000)
            r = tune_segments(uw, a[:m], b[:m], DELTA, reps=1)
        tuned = {"kernel": r.kernel, "config": r.best, "default_ms": r.default_ms, "best_ms": r.best_ms,
                 "configs_tried": len(r.table)}
    for _ in range(args.warmup):
        work.gpu(uw, a, b)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats = []
    stream = torch.cuda.current_stream(dev)
    with ClockSampler(local) as clk:
        barrier()
        for i in range(args.steps):
            flush.zero_()                      # L2 flush between timed steps (not timed)
            ev[i][0].record(stream)
            f = work.gpu(uw, a, b)
            ev[i][1].record(stream)
            stats.append(uw.last_stats())      # synchronises; outside the event pair
        barrier()
    step_ms = [s.elapsed_time(e) for s, e in ev]
    my_ms = sum(step_ms)
    my_checks = sum(s["reference_checks"] for s in stats)
    tot_ms, tot_checks = max_time_sum_units(my_ms, my_checks, ws, dev)
    value = tot_checks / (tot_ms / 1e3)

    # both kinds of BVH node box on the same batch: time per step and the tests they take
    boxes = {}
    bk = 1 if args.workload == "segments" else 0
    default_kind = uw.get_node_boxes(bk)
    for kind in ("aligned", "oriented"):
        uw.set_node_boxes(kind, bk)
        for _ in range(2):
            work.gpu(uw, a, b)
        bms, bst = [], None
        for i in range(min(args.steps, 5)):
            flush.zero_()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            fb = work.gpu(uw, a, b)
            s1.record(stream)
            bst = uw.last_stats()
            bms.append(s0.elapsed_time(s1))
        if not torch.equal(fb, f):
            raise RuntimeError("%s node boxes changed the results" % kind)
        boxes[kind] = {"ms_per_step": sum(bms) / len(bms), "node_tests": bst["node_tests"],
                       "leaf_tests": bst["leaf_tests"], "fp64_retests": bst["retests"],
                       "traverse_ms": bst["traverse_ms"]}
    uw.set_node_boxes(default_kind, bk)
    boxes["default"] = default_kind

    # the same query replayed as one CUDA graph (graph mode: no host synchronisation inside the step)
    graph_ms = None
    if args.workload == "segments":
        from puzzletunneldiscovery_gb300.autotune import SegmentGraph
        g = SegmentGraph(uw, a, b, DELTA)
        g.replay()
        gms = []
        for i in range(args.steps):
            flush.zero_()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            gout = g.replay()
            s1.record(stream)
            torch.cuda.synchronize(dev)
            gms.append(s0.elapsed_time(s1))
        if not torch.equal(gout, f):
            raise RuntimeError("graph replay changed first-contact steps")
        graph_ms = sum(gms) / len(gms)
        del g

    # end to end through the public host-array API with pinned host buffers: every
    # step copies its inputs in and its results out inside the timed region
    ha = torch.from_numpy(work.q0).pin_memory()
    hb = torch.from_numpy(work.q1).pin_memory() if work.q1 is not None else None
    checks_per_step = stats[0]["reference_checks"]   # the same batch as the timed device steps
    e2e_ms, e2e_checks = 0.0, 0
    barrier()
    for i in range(args.steps):
        flush.zero_()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        hout = work.gpu_host(uw, ha, hb)
        s1.record(stream)
        torch.cuda.synchronize(dev)
        e2e_ms += s0.elapsed_time(s1)
        e2e_checks += checks_per_step
    if not torch.equal(hout.to(dev), f):
        raise RuntimeError("host-array path disagrees with the device path")
    e2e_ms, e2e_checks = max_time_sum_units(e2e_ms, e2e_checks, ws, dev)
    e2e_value = e2e_checks / (e2e_ms / 1e3)

    if rank != 0:
        if ws > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    # roofline of the dominant (traversal) kernel
    roof = traversal_roofline(stats, work.bytes_in() + work.bytes_out(), args.n, args.workload,
                              uw.get_node_boxes(1 if args.workload == "segments" else 0))
    fc = f.cpu().numpy()
    cpu, parity = None, None
    if ws == 1 and not args.no_cpu_baseline:
        cpu, parity = cpu_baseline(work, fc, target_s=args.cpu_seconds)
    sur = None
    if args.workload == "segments" and not args.no_surrogate_arm:
        # the second half of the metric: verified free samples per second, surrogate-guided
        # against plain, on the same meshes (config: 50M training labels, 200M candidates, top 10 %)
        sur = surrogate_measure(args, local, rank, WORKLOADS["surrogate"][2], steps=min(args.steps, 10),
                                warmup=min(args.warmup, 3), with_cpu=(ws == 1 and not args.no_cpu_baseline),
                                e2e=False)
        sur = surrogate_summary(sur)
    last = stats[-1]
    if args.workload == "segments":
        config = {"workload": "segments_first_contact/interlocking_tori",
                  "meshes": "torus R=1 r=0.25 64x32 (4096 tris) x2, interlocked",
                  "n_segments_per_gpu": args.n, "verify_delta": DELTA, "mode": "transit_state_to"}
        extra = {"segments_per_s": args.n * ws / (tot_ms / args.steps / 1e3),
                 "free_fraction": float((fc == -1).mean()),
                 "detailed_chunk_fraction": last["detailed_chunks"] / max(1, last["work_items"])}
    else:
        config = {"workload": "is_valid_state/perforated_plate_vs_torus_knot",
                  "meshes": "plate 400x400 grid over [-2,2]^2 with 25 holes (%d tris), (2,3) knot 256x16 (8192 tris)"
                            % len(Fe),
                  "n_states_per_gpu": args.n}
        extra = {"free_fraction": float(fc.astype(bool).mean())}
    config.update({"l2": "flushed (256 MB write) between timed steps; per-step working set > L2",
                   "parallelism": "replicas" if ws == 1 else "shard-per-rank (weak)", "bvh": BVH_KIND})
    line = {"metric": work.metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 traversal + f64 state math/re-tests",
            "data": "synthetic (seeded; no published data set for this path)",
            "config": config, "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(work.bytes_in() * ws),
                    "d2h_bytes_per_step": int(work.bytes_out() * ws)},
            "clocks": clk.summary(),
            # the library's own count per query (segments: bounds, set-up, rounds, anchors and
            # traversal per round phase, re-test, finalise; states: traversal, re-test; CUB's scans
            # and sorts not counted), summed over the timed steps
            "gpu_launches": int(sum(st["kernel_launches"] for st in stats)),
            "detail": dict({"mismatches": parity["mismatches"] if parity else None,
                            "mismatch_sample": parity["mismatch_sample"] if parity else 0,
                            "parity": parity,
                            "reference_checks_per_step": tot_checks / args.steps,
                            "gpu_queries_per_step": last["queries"], "node_tests": last["node_tests"],
                            "leaf_tests": last["leaf_tests"], "fp64_retests": last["retests"],
                            "fp64_retest_rate_per_leaf": last["retests"] / max(1, last["leaf_tests"]),
                            "inline_retests": last["inline_retests"], "retest_ms": last["retest_ms"],
                            "step_ms": step_ms, "autotune": tuned, "graph_replay_ms_per_step": graph_ms,
                            "node_boxes": boxes},
                           **extra)}
    if sur is not None:
        line["detail"]["surrogate"] = sur
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    bad = parity["mismatches"] if parity else 0
    if sur is not None:
        bad += (sur["mismatches"] or 0) + sur["false_free_accepted"] + (sur["false_free_oracle"] or 0)
    if bad:
        print("verdict mismatches against the oracle: %d" % bad, file=sys.stderr)
        sys.exit(3)


def traversal_roofline(stats, io_bytes, n_units, workload, boxes="aligned"):
    """Roofline record of the traversal kernel.  The algorithmic DRAM bytes are
    the queries' inputs and results; the BVH nodes and triangles the tests read
    are L2-resident, so those bytes are reported apart (cache_served), and the
    binding limit, SM instruction issue, is given with its measured fraction
    from the committed ncu capture."""
    trav_ms = sum(s["traverse_ms"] for s in stats) / len(stats)
    node = sum(s["node_tests"] for s in stats) / len(stats)
    leaf = sum(s["leaf_tests"] for s in stats) / len(stats)
    sec = trav_ms / 1e3
    peak, peak_kind = _peaks()
    achieved = io_bytes / sec / 1e9
    seg = workload != "plate"
    # DRAM traffic per unit from the committed capture of this workload's kernel (none for the
    # narrow-passage validation, whose segments run on the plate meshes); issue utilisation from
    # the capture of the same kernel
    prof = "k_segments_traffic.txt" if seg else "k_states_plate_traffic.txt"
    per_unit = None
    if workload == "segments":
        per_unit = _profile_value(prof, "dram_bytes_per_segment")
    elif workload == "plate":
        per_unit = _profile_value(prof, "dram_bytes_per_state")
    traffic = per_unit * n_units if per_unit is not None else None
    issue = _profile_value(prof, "smsp_issue_active_pct")
    node_pair = BYTES_NODE_PAIR_OBB if boxes == "oriented" else BYTES_NODE_PAIR
    cache_bytes = node * node_pair + leaf * BYTES_LEAF_PAIR
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic,
            "traffic_frac": (traffic / sec / 1e9 / peak) if traffic is not None else None,
            "kernel": "k_segments" if seg else "k_states", "kernel_ms": trav_ms, "peak_source": peak_kind,
            "algorithmic_bytes": io_bytes,
            "algorithmic_bytes_what": "the queries' inputs and results (%s)" %
                                      ("two 56 B states in, a 4 B step out" if seg else "a 56 B state in, 1 B out"),
            "limiter": "SM instruction issue: BVH nodes and triangles are L2-resident, DRAM moves only the queries",
            "limiter_frac": issue / 100.0 if issue is not None else None,
            "limiter_source": "smsp__issue_active of the committed ncu capture (profiles/)",
            "cache_served": {"bytes": cache_bytes, "achieved": cache_bytes / sec / 1e9, "unit": "GB/s",
                             "what": "node-pair tests x %d B + leaf tests x %d B, read from L1/L2"
                                     % (node_pair, BYTES_LEAF_PAIR)}}


def surrogate_measure(args, local, rank, n, steps, warmup, with_cpu, e2e=True):
    """Learned proposal on the interlocking tori: train on exact labels, then
    per step rank `n` uniform candidates with the network, check the top
    fraction exactly and count the verified free samples.  The plain arm
    checks every candidate exactly.  Returns every figure of the measurement;
    with_cpu adds the oracle on the host cores over a sample of the same
    candidates, whose verdicts are compared with the plain arm's, and the
    oracle's re-check of a sample of the accepted set."""
    import torch

    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import surrogate as S

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    Ve, Fe, Vr, Fr = _meshes("surrogate")
    uw = pw.UnitWorld(local)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.set_bvh(BVH_KIND)
    uw.angleModel(0.0, 0.0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1000 + rank)
    draw = lambda m: S.uniform_states_device(m, -2.0, 2.0, uw.scene_scale, gen, dev)  # noqa: E731
    stream = torch.cuda.current_stream(dev)

    # training on exact labels (timed as its own phase)
    net = S.Surrogate(local, seed=rank)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    t0.record(stream)
    rep = S.train_online(uw, net, draw, args.train_labels, batch=65536, lr=1e-3, log_every=100)
    t1.record(stream)
    torch.cuda.synchronize(dev)
    train_ms = t0.elapsed_time(t1)

    cand = draw(n)                            # resident candidates (not timed)
    prob = torch.empty(n, dtype=torch.float32, device=dev)
    # the states kernel's node boxes, picked on a sample of the candidates
    from puzzletunneldiscovery_gb300.autotune import pick_node_boxes
    boxes = pick_node_boxes(uw, states=cand[: 1 << 22])
    # exact labels of a 4M sample: precision / recall of the network as a free-space predictor
    sample = cand[: 1 << 22]
    exact = uw.is_valid_states(sample)
    prec, rec = S.precision_recall(net.predict(sample), exact)
    net.check()
    m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def guided(frac=args.top_frac):
        net.score(cand, out=prob)
        m1.record(stream)
        sel = S.select_top(prob, cand, int(round(frac * n)))
        ok = uw.is_valid_states(sel)
        return sel, ok

    def plain():
        return uw.is_valid_states(cand)

    for _ in range(warmup):
        guided()
        plain()
    torch.cuda.synchronize(dev)
    g_ms, p_ms, mlp_ms, g_free, p_free, g_checked, false_free = [], [], [], 0, 0, 0, 0
    accepted = None
    with ClockSampler(local) as clk:
        for i in range(steps):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            m0.record(stream)
            sel, ok = guided()
            nfree = ok.sum()
            s1.record(stream)
            torch.cuda.synchronize(dev)
            g_ms.append(s0.elapsed_time(s1))
            mlp_ms.append(m0.elapsed_time(m1))
            g_free += int(nfree)
            g_checked += int(sel.shape[0])
            if i == 0:
                # every accepted sample was checked exactly; re-check the accepted set once
                accepted = sel[ok]
                false_free = int((~uw.is_valid_states(accepted)).sum())
            s0.record(stream)
            okp = plain()
            nfree = okp.sum()
            s1.record(stream)
            torch.cuda.synchronize(dev)
            p_ms.append(s0.elapsed_time(s1))
            p_free += int(nfree)
    value = g_free / (sum(g_ms) / 1e3)
    plain_value = p_free / (sum(p_ms) / 1e3)
    # the same pipeline at larger checked fractions (one timed step each)
    sweep = {}
    for frac in args.sweep:
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        s0.record(stream)
        m0.record(stream)
        sel, ok = guided(frac)
        nfree = ok.sum()
        s1.record(stream)
        torch.cuda.synchronize(dev)
        ms = s0.elapsed_time(s1)
        sweep["%.2f" % frac] = {"verified_free_per_s": int(nfree) / (ms / 1e3), "ms": ms,
                                "precision": int(nfree) / max(1, sel.shape[0]),
                                "over_plain": int(nfree) / (ms / 1e3) / plain_value}

    out = {"value": value, "plain_value": plain_value, "n": n, "steps": steps, "warmup": warmup,
           "top_frac": args.top_frac,
           "g_ms": g_ms, "p_ms": p_ms, "g_free": g_free, "p_free": p_free, "g_checked": g_checked,
           "precision": prec, "recall": rec, "false_free": false_free, "train_ms": train_ms, "rep": rep,
           "sweep": sweep, "clocks": clk.summary(), "e2e": None, "cpu": None, "parity": None, "node_boxes": boxes}

    if e2e:
        # end to end: candidates from pinned host memory, accepted states back to the host
        e2e_n = min(args.e2e_n, n)
        hc = cand[:e2e_n].cpu().pin_memory()
        e2e_ms, e2e_free, h2d, d2h = 0.0, 0, 0, 0
        for i in range(steps):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            dc = hc.to(dev, non_blocking=True)
            pr = net.score(dc)
            sel = S.select_top(pr, dc, int(round(args.top_frac * dc.shape[0])))
            acc = sel[uw.is_valid_states(sel)]
            hacc = acc.cpu()
            s1.record(stream)
            torch.cuda.synchronize(dev)
            e2e_ms += s0.elapsed_time(s1)
            e2e_free += hacc.shape[0]
            h2d, d2h = hc.numel() * 8, hacc.numel() * 8
        out["e2e"] = {"value": e2e_free / (e2e_ms / 1e3), "unit": "samples/s", "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h, "candidates_per_step": e2e_n}

    mlp_kernel_ms = sum(mlp_ms) / len(mlp_ms)
    achieved = MLP_FLOP_PER_ROW * n / (mlp_kernel_ms / 1e3) / 1e12
    peak, peak_kind = _bf16_peak()
    tpr = _profile_value("k_mlp_forward_tc_traffic.txt", "dram_bytes_per_row")
    out["mlp_ms"] = mlp_kernel_ms
    out["roof"] = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                   "frac": achieved / peak, "traffic": tpr * n if tpr is not None else None,
                   "kernel": "k_mlp_forward_tc", "kernel_ms": mlp_kernel_ms, "peak_source": peak_kind,
                   "algorithmic_flop": MLP_FLOP_PER_ROW * n}
    if with_cpu:
        okp_host = okp.cpu().numpy()
        out["cpu"], out["parity"] = _cpu_plain_sampling(cand, okp_host, args.cpu_seconds)
        # the oracle re-checks a sample of the accepted set: none may be in collision
        from oracle import oracle as O
        ow = O.OracleWorld(Ve, Fe, Vr, Fr)
        acc = accepted[:200_000].cpu().numpy()
        out["false_free_oracle"] = int((~ow.is_valid(acc, nthreads=os.cpu_count() or 1)).sum())
        out["false_free_oracle_sample"] = int(acc.shape[0])
    return out


def surrogate_summary(m):
    """The surrogate measurement as a compact dict (the headline line's detail)."""
    b = m["sweep"]
    return {"metric": WORKLOADS["surrogate"][0], "unit": "samples/s",
            "config": {"candidates_per_step": m["n"], "top_fraction": m["top_frac"], "train_labels": m["rep"].labels,
                       "batch": 65536, "lr": 1e-3, "network": "9 -> 256x4 SiLU -> 1 sigmoid, BF16"},
            "guided_verified_free_per_s": m["value"], "plain_verified_free_per_s": m["plain_value"],
            "guided_over_plain": m["value"] / m["plain_value"],
            "guided_ms_per_step": sum(m["g_ms"]) / len(m["g_ms"]),
            "plain_ms_per_step": sum(m["p_ms"]) / len(m["p_ms"]), "mlp_ms_per_step": m["mlp_ms"],
            "steps": m["steps"], "precision_at_0.5": m["precision"], "recall_at_0.5": m["recall"],
            "precision_top_fraction": m["g_free"] / max(1, m["g_checked"]),
            "false_free_accepted": m["false_free"], "false_free_oracle": m.get("false_free_oracle"),
            "false_free_oracle_sample": m.get("false_free_oracle_sample", 0),
            "mismatches": m["parity"]["mismatches"] if m["parity"] else None,
            "mismatch_sample": m["parity"]["mismatch_sample"] if m["parity"] else 0,
            "train_ms": m["train_ms"], "roofline": m["roof"], "cpu_baseline": m["cpu"],
            "top_fraction_sweep": {k: v["over_plain"] for k, v in b.items()}, "clocks": m["clocks"],
            "node_boxes": m["node_boxes"]}


def run_surrogate(args):
    """--workload surrogate: the learned proposal's own line."""
    ws, rank, local = _dist_env()
    m = surrogate_measure(args, local, rank, args.n, args.steps, args.warmup,
                          with_cpu=(ws == 1 and not args.no_cpu_baseline))
    if rank != 0:
        return
    rep = m["rep"]
    value, plain_value = m["value"], m["plain_value"]
    line = {"metric": WORKLOADS["surrogate"][0], "value": value, "unit": "samples/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(m["g_ms"]) / len(m["g_ms"]),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 network (f32 accumulate) + f32/f64 exact checks",
            "data": "synthetic (seeded uniform states on the device)",
            "config": {"workload": "surrogate_guided_sampling/interlocking_tori", "candidates_per_step": args.n,
                       "top_fraction": args.top_frac, "train_labels": args.train_labels, "batch": 65536,
                       "lr": 1e-3, "network": "9 -> 256x4 SiLU -> 1 sigmoid, BF16",
                       "l2": "per-step working set (11 GB of candidates) > L2",
                       "parallelism": "replicas" if ws == 1 else "independent replicas"},
            "roofline": m["roof"], "cpu_baseline": m["cpu"], "e2e": m["e2e"], "clocks": m["clocks"],
            # per guided step: network scores, 3 histogram passes and the compaction of the
            # exact top-k, the traversal and re-test of the selected states
            "gpu_launches": 7 * args.steps,
            "detail": {"mismatches": m["parity"]["mismatches"] if m["parity"] else None,
                       "mismatch_sample": m["parity"]["mismatch_sample"] if m["parity"] else 0,
                       "parity": m["parity"],
                       "plain_verified_free_per_s": plain_value, "guided_over_plain": value / plain_value,
                       "plain_ms_per_step": sum(m["p_ms"]) / len(m["p_ms"]),
                       "guided_ms_per_step": sum(m["g_ms"]) / len(m["g_ms"]),
                       "mlp_ms_per_step": m["mlp_ms"], "mlp_rows_per_s": args.n / (m["mlp_ms"] / 1e3),
                       "checked_per_step": m["g_checked"] / args.steps,
                       "precision_top_fraction": m["g_free"] / max(1, m["g_checked"]),
                       "plain_free_fraction": m["p_free"] / (args.n * args.steps),
                       "precision_at_0.5": m["precision"], "recall_at_0.5": m["recall"],
                       "false_free_accepted": m["false_free"], "false_free_oracle": m.get("false_free_oracle"),
                       "false_free_oracle_sample": m.get("false_free_oracle_sample", 0),
                       "train_ms": m["train_ms"], "train_steps": rep.steps,
                       "train_labels_per_s": rep.labels / (m["train_ms"] / 1e3),
                       "train_loss_first_last": [rep.losses[0][1], rep.losses[-1][1]] if rep.losses else None,
                       "top_fraction_sweep": m["sweep"], "node_boxes": m["node_boxes"]}}
    print(json.dumps(line), flush=True)
    bad = (line["detail"]["mismatches"] or 0) + m["false_free"] + (m.get("false_free_oracle") or 0)
    if bad:
        print("verdict mismatches against the oracle: %d" % bad, file=sys.stderr)
        sys.exit(3)


def run_narrow(args):
    """Narrow-passage search on the plate / torus-knot meshes: per step, every
    root is expanded 64 times, expansions that carry the knot through the
    plate plane are ranked by the network (guided) or drawn at random (plain),
    and the top k per round are validated exactly as segments in one graph
    replay.  Value = escapes (exactly free crossing motions) per second."""
    import torch

    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import narrow as N
    from puzzletunneldiscovery_gb300 import surrogate as S

    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    Ve, Fe, Vr, Fr = _meshes("narrow")
    uw = pw.UnitWorld(local)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.set_bvh(BVH_KIND)
    uw.angleModel(0.0, 0.0)
    s = uw.scene_scale
    lo, hi = Ve.min(0) - 0.5, Ve.max(0) + 0.5
    gen = torch.Generator(device=dev)
    gen.manual_seed(2000 + rank)
    roots = N.draw_free_roots(uw, args.n, lo, hi, gen)
    probes = N.centre_line_probes(uw, 256, 16, every=8)
    extent = float(np.abs(Ve[:, :2]).max()) * s
    net = S.Surrogate(local, seed=rank)
    search = N.NarrowPassageSearch(uw, net, probes, 0.0, extent, per_root=64, sigma_t=0.05, sigma_rot=0.1,
                                   k=args.narrow_k, verify_delta=DELTA, retrain_labels=10_000_000, seed=rank)
    # initial training: exact labels of the crossing expansions of separate free roots
    t0 = time.perf_counter()
    warm_roots = N.draw_free_roots(uw, min(args.n, 1 << 21), lo, hi, gen)
    train_steps = search.pretrain(warm_roots, args.narrow_train_labels)
    torch.cuda.synchronize(dev)
    train_s = time.perf_counter() - t0
    # node boxes of both kernels, picked on crossing candidates of separate roots (the
    # motions the searches validate, and their endpoints, which label the network)
    from puzzletunneldiscovery_gb300.autotune import pick_node_boxes
    R = warm_roots[: 1 << 18]
    ends = N.expand(R, 64, 0.05 * s, 0.1, 12345)
    ci = torch.nonzero(N.crossings(R, ends, 64, torch.from_numpy(np.ascontiguousarray(probes)).to(dev), 0.0,
                                   extent)).flatten()[:65536]
    boxes = pick_node_boxes(uw, states=ends.index_select(0, ci),
                            segments=(R.index_select(0, ci // 64).contiguous(), ends.index_select(0, ci).contiguous()),
                            verify_delta=DELTA, mode=1)
    # the plain arm gets its own world, so that the two searches' captured graphs
    # never invalidate each other's scratch
    uw_plain = pw.UnitWorld(local)
    uw_plain.load_env_mesh(Ve, Fe)
    uw_plain.load_robot_mesh(Vr, Fr)
    uw_plain.scaleToUnit()
    uw_plain.set_bvh(BVH_KIND)
    uw_plain.angleModel(0.0, 0.0)
    uw_plain.set_node_boxes(boxes["states"], 0)
    uw_plain.set_node_boxes(boxes["segments"], 1)
    plain = N.NarrowPassageSearch(uw_plain, None, probes, 0.0, extent, per_root=64, sigma_t=0.05, sigma_rot=0.1,
                                  k=args.narrow_k, verify_delta=DELTA, seed=rank)
    for _ in range(args.warmup):
        search.run(roots, guided=True)
        plain.run(roots, guided=False)
    g_reps, p_reps = [], []
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            g_reps.append(search.run(roots, guided=True, keep_escapes=(i == 0), keep_validated=(i == 0)))
            p_reps.append(plain.run(roots, guided=False, keep_validated=(i == 0)))
    g_esc = sum(r.escapes for r in g_reps)
    g_s = sum(r.seconds for r in g_reps)
    p_esc = sum(r.escapes for r in p_reps)
    p_s = sum(r.seconds for r in p_reps)
    value = g_esc / g_s
    plain_value = p_esc / p_s
    # every escape of the first guided step again, outside the graph: false-free must be 0
    false_free = 0
    for frm, to in g_reps[0].escape_states:
        if frm.shape[0]:
            false_free += int((uw.first_contact_steps(frm, to, DELTA, 1) != -1).sum())
    # end to end: roots from pinned host memory, escapes back to the host
    hroots = roots.cpu().pin_memory()
    e2e_esc, e2e_s, d2h = 0, 0.0, 0
    for i in range(args.steps):
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        droots = hroots.to(dev, non_blocking=True)
        r = search.run(droots, guided=True, keep_escapes=True)
        host = [(f.cpu(), t_.cpu()) for f, t_ in r.escape_states]
        torch.cuda.synchronize(dev)
        e2e_s += time.perf_counter() - t
        e2e_esc += r.escapes
        d2h = sum(f.numel() * 8 * 2 for f, _ in host)
    if rank != 0:
        return
    last = g_reps[-1]
    # roofline of the dominant kernel: the first guided round's validated motions once more as a
    # direct call (the search replays them as a graph), with the traversal's counters and events
    gf, gt, gcodes = g_reps[0].validated_states
    uw.first_contact_steps(gf, gt, DELTA, 1)
    st = uw.last_stats()
    roof = traversal_roofline([st], gf.shape[0] * (2 * 56 + 4), gf.shape[0], "narrow", uw.get_node_boxes(1))
    roof["kernel_share"] = "exact validation is %.0f %% of a guided round" % (
        100.0 * st["traverse_ms"] * last.rounds / max(1e-9, 1e3 * g_reps[-1].seconds))
    cpu, parity = None, None
    if ws == 1 and not args.no_cpu_baseline:
        cpu, parity = _cpu_plain_narrow(p_reps[0].validated_states, args.cpu_seconds)
    line = {"metric": WORKLOADS["narrow"][0], "value": value, "unit": "escapes/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * g_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 network (f32 accumulate) + f32/f64 exact segment checks",
            "data": "synthetic (seeded free roots over the plate's box padded by 0.5)",
            "config": {"workload": "narrow_passage_search/perforated_plate_vs_torus_knot", "roots": args.n,
                       "expansions_per_root": 64, "sigma_t": 0.05, "sigma_rot": 0.1,
                       "validated_per_round": args.narrow_k, "roots_per_round": 1 << 20,
                       "verify_delta": DELTA, "initial_train_labels": args.narrow_train_labels,
                       "score": "min of the network's logits at the motion's midpoint and endpoint",
                       "retrain_every_labels": 10_000_000,
                       "escape": "an exactly free segment along which a knot centre-line point crosses the "
                                 "plate plane inside the plate (hence through a hole)",
                       "l2": "per-step working set (roots and 64x expansions, GBs) > L2",
                       "parallelism": "replicas"},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_esc / e2e_s, "unit": "escapes/s", "h2d_bytes_per_step": int(hroots.numel() * 8),
                    "d2h_bytes_per_step": int(d2h)},
            "clocks": clk.summary(),
            # this project's kernels per guided round: crossing filter 1, network scores 2, the
            # replayed validation graph 7 (bounds, set-up, anchors, rounds, traversal, re-test,
            # finalise; its CUB scan and sort kernels not counted), endpoint labels 2 (traversal, re-test)
            "gpu_launches": 12 * sum(r.rounds for r in g_reps),
            "detail": {"mismatches": parity["mismatches"] if parity else None,
                       "mismatch_sample": parity["mismatch_sample"] if parity else 0, "parity": parity,
                       "node_boxes": boxes,
                       "plain_escapes_per_s": plain_value, "guided_over_plain": value / max(plain_value, 1e-12),
                       "guided_yield": g_esc / max(1, sum(r.validated for r in g_reps)),
                       "plain_yield": p_esc / max(1, sum(r.validated for r in p_reps)),
                       "escapes_per_step": g_esc / args.steps, "plain_escapes_per_step": p_esc / args.steps,
                       "crossing_fraction": last.crossing / max(1, last.candidates),
                       "validated_per_step": last.validated, "rounds_per_step": last.rounds,
                       "false_free_escapes": false_free, "retrains": sum(r.retrains for r in g_reps),
                       "initial_train_s": train_s, "initial_train_steps": train_steps,
                       "plain_ms_per_step": 1e3 * p_s / args.steps}}
    print(json.dumps(line), flush=True)
    bad = (parity["mismatches"] if parity else 0) + false_free
    if bad:
        print("verdict mismatches against the oracle: %d" % bad, file=sys.stderr)
        sys.exit(3)


def _cpu_plain_narrow(validated, target_s):
    """The plain narrow-passage search's exact validations on the host cores: the
    oracle's is_valid_transition over the motions of the plain search's first
    round (grown until it takes about target_s), escapes per second, and its
    first-contact codes compared with the GPU's.  Returns (cpu_baseline, parity)."""
    from oracle import oracle as O
    O.build()
    Ve, Fe, Vr, Fr = _meshes("narrow")
    ow = O.OracleWorld(Ve, Fe, Vr, Fr)
    cores = os.cpu_count() or 1
    frm, to, codes = (t.cpu().numpy() for t in validated)
    n = 256
    while True:
        n = min(n, frm.shape[0])
        t0 = time.perf_counter()
        first, _ = ow.segments_first_contact(frm[:n], to[:n], DELTA, mode=1, nthreads=cores)
        dt = time.perf_counter() - t0
        if dt >= target_s or n >= frm.shape[0]:
            break
        n = max(n * 2, int(n * target_s / max(dt, 1e-3) * 1.1))
    esc = int((first == -1).sum())
    cpu = {"value": esc / dt, "unit": "escapes/s", "cores": cores, "kind": "port",
           "sample": "the first %d motions the plain search validated in its first round (is_valid_transition, "
                     "%d escapes, %.1f s; expansion and the crossing filter not counted)" % (n, esc, dt)}
    parity = {"mismatches": int((first != codes[:n]).sum()), "mismatch_sample": int(n),
              "compared": "is_valid_transition first-contact code of every motion",
              "sample": "the CPU-baseline sample, against the plain search's graph-replayed validation"}
    return cpu, parity


def _keyconf_half_angles(spins):
    """Cosine and sine of half of each enumFreeConfiguration spin angle i * 2 pi / spins."""
    delta = 2 * math.pi / float(spins)
    half = [0.5 * (i * delta) for i in range(spins)]
    return [math.cos(h) for h in half], [math.sin(h) for h in half]


def _surface_pairs(V, F, Vr, Fr, n, rng):
    """n (robot point, robot normal, env point, env normal) surface samples: a
    triangle drawn by area, a uniform point on it, the face's unit normal."""
    def draw(V, F):
        a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
        nrm = np.cross(b - a, c - a)
        area = np.linalg.norm(nrm, axis=1)
        t = rng.choice(len(F), n, p=area / area.sum())
        u, v = rng.random(n), rng.random(n)
        flip = u + v > 1
        u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
        pts = a[t] + u[:, None] * (b[t] - a[t]) + v[:, None] * (c[t] - a[t])
        return pts, nrm[t] / area[t][:, None]
    rp, rn = draw(Vr, Fr)
    ep, en = draw(V, F)
    return rp, rn, ep, en


class RowJob:
    """One of the row workloads (is_disentangled, contact enumeration, key
    configurations, touch sampling) on the interlocking tori: the batch of one
    step, the GPU call through the public API, the oracle on a sample and the
    comparison of their results."""

    def __init__(self, name, uw, n, seed):
        import torch
        self.name, self.uw, self.n = name, uw, n
        self.launches = 0   # kernels the library reports for the contact enumerations made
        s = uw.scene_scale
        rng = np.random.default_rng(3000 + seed)
        self.dev = uw._device
        self.device_timed = name == "disentangled"
        if name == "disentangled":
            self.q = W.uniform_states(n, -2.0, 2.0, s, seed=seed)
            self.a = torch.from_numpy(self.q).to(self.dev)
            self.units, self.unit = n, "checks/s"
        elif name == "contacts":
            q = W.uniform_states(8 * n, -0.6, 0.6, s, seed=seed)
            hit = ~uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
            self.q = q[hit][:n]
            self.n = self.q.shape[0]
            self.units, self.unit = self.n, "states/s"
        elif name == "keyconf":
            Ve, Fe = uw._cd(0)
            Vr, Fr = uw._cd(1)
            self.pairs = _surface_pairs(Ve, Fe, Vr, Fr, n, rng)
            self.units, self.unit = n * KEYCONF_SPINS, "checks/s"
        elif name == "visibility":
            q = W.uniform_states(4 * n, -2.0, 2.0, s, seed=seed)
            ok = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
            self.keys = np.ascontiguousarray(q[ok][:n])
            self.n = self.keys.shape[0]
            self.units, self.unit = self.n * (self.n - 1) // 2, "pairs/s"
        else:
            q = W.uniform_states(4 * n, -2.0, 2.0, s, seed=seed)
            ok = uw.is_valid_states(torch.from_numpy(q)).cpu().numpy()
            self.keys = q[ok][:n]
            self.units, self.unit = self.keys.shape[0] * TOUCH_PER_KEY, "segments/s"
        self.seed = seed

    def gpu(self):
        """One step through the public API; returns the step's result.  Counts the
        library's kernel launches (its own report after each query, plus the
        world-free state generators)."""
        from puzzletunneldiscovery_gb300 import sampling as SP
        uw = self.uw
        if self.name == "disentangled":
            res = uw.is_disentangled_states(self.a)
        elif self.name == "contacts":
            res = uw.intersecting_segments_batch(self.q, flat=True)
        elif self.name == "keyconf":
            rp, rn, ep, en = self.pairs
            res = SP.enum_free_configurations(uw, rp, rn, ep, en, KEYCONF_MARGIN, KEYCONF_SPINS, only_median=True)
            self.launches += 1                                       # pw_keyconf_states
        elif self.name == "visibility":
            res = self._visibility(uw)
            return res
        else:
            res, self.to = SP.calc_touch_batch(uw, self.keys, TOUCH_PER_KEY, uw.recommended_cres,
                                               np.random.default_rng(4000 + self.seed))
            self.launches += 1                                       # pw_touch_targets
        self.launches += uw.last_stats()["kernel_launches"]
        return res

    def _visibility(self, uw):
        """calculate_visibility_matrix in chunks of pairs, each chunk's launches counted."""
        out = uw.calculate_visibility_matrix(self.keys, True, VIS_DELTA)
        # one segment query per chunk of 2^22 pairs; the last one's report stands for each
        chunks = -(-self.units // uw._PAIR_CHUNK)
        self.launches += chunks * uw.last_stats()["kernel_launches"]
        return out

    def cpu(self, ow, m, threads):
        """(units, seconds, result) of the oracle on the first m units of the step."""
        from puzzletunneldiscovery_gb300 import sampling as SP
        t0 = time.perf_counter()
        if self.name == "disentangled":
            res = ow.is_disentangled(self.q[:m], nthreads=threads)
            units = m
        elif self.name == "contacts":
            import concurrent.futures as cf
            with cf.ThreadPoolExecutor(max_workers=threads) as ex:
                res = list(ex.map(ow.intersecting_segments, self.q[:m]))
            units = m
        elif self.name == "visibility":
            lo, hi = np.triu_indices(m, 1)
            codes, _ = ow.segments_first_contact(self.keys[lo], self.keys[hi], VIS_DELTA, mode=1, nthreads=threads)
            res = np.zeros((m, m), np.int8)
            res[lo, hi] = res[hi, lo] = (codes == -1)
            units = lo.shape[0]
        elif self.name == "keyconf":
            from oracle import oracle as O
            rp, rn, ep, en = (x[:m] for x in self.pairs)
            hc, hs = _keyconf_half_angles(KEYCONF_SPINS)
            qs = O.keyconf_states(rp, rn, ep, en, KEYCONF_MARGIN, hc, hs, nthreads=threads)
            valid = ow.is_valid(qs.reshape(-1, 7), nthreads=threads).reshape(m, KEYCONF_SPINS)
            res = O.free_spins(qs, valid, True)
            units = m * KEYCONF_SPINS
        else:
            k = m * TOUCH_PER_KEY
            frm = np.repeat(self.keys[:m], TOUCH_PER_KEY, axis=0)
            res, _ = ow.segments_first_contact(frm, self._targets(k), self.uw.recommended_cres, mode=0,
                                               nthreads=threads)
            units = k
        return units, time.perf_counter() - t0, res

    def _targets(self, k):
        """The first k touch targets of the last step, on the host."""
        to = self.to[:k]
        return to.cpu().numpy() if hasattr(to, "cpu") else to

    def mismatches(self, ow, gpu_res, cpu_res, m):
        """Results of the first m units that differ from the oracle's."""
        if self.name == "disentangled":
            return int((gpu_res[:m].cpu().numpy() != cpu_res).sum())
        if self.name == "contacts":
            bad = 0
            b, e, mg, p, off = gpu_res
            rows = [(b[o0:o1], e[o0:o1], mg[o0:o1], p[o0:o1]) for o0, o1 in zip(off[:m], off[1:m + 1])]
            for (b, e, mg, p), (b2, e2, mg2, p2, _) in zip(rows, cpu_res):
                same = p.shape == p2.shape and (p == p2).all() and (b == b2).all() and (e == e2).all() \
                    and (mg == mg2).all()
                bad += 0 if same else 1
            return bad
        if self.name == "keyconf":
            return sum(0 if np.array_equal(x, y) else 1 for x, y in zip(gpu_res[:m], cpu_res))
        if self.name == "visibility":
            lo, hi = np.triu_indices(m, 1)
            return int((gpu_res[:m, :m][lo, hi] != cpu_res[lo, hi]).sum())
        # touch: the GPU's tuples against the oracle's first contacts (done = no contact), and the
        # full tuples of the first 256 segments against the oracle's transit loop
        k = m * TOUCH_PER_KEY
        lf, st, done, lt, tt = gpu_res
        bad = int((done[:k].astype(bool) != (cpu_res == -1)).sum())
        frm = np.repeat(self.keys[:m], TOUCH_PER_KEY, axis=0)
        to = self._targets(min(k, 256))
        for i in range(min(k, 256)):
            (wl, ws_, wd, wlt, wtt), _, _ = ow.transit_state_to_with_contact(frm[i], to[i],
                                                                              self.uw.recommended_cres)
            same = (lf[i] == wl).all() and (st[i] == ws_).all() and bool(done[i]) == wd and lt[i] == wlt \
                and tt[i] == wtt
            bad += 0 if same else 1
        return bad


def run_rows(args):
    """--workload disentangled | contacts | keyconf | touch: one row of the path
    through the public API, timed per step; the oracle on a sample of the same
    step on the host cores, with its results compared."""
    import torch

    import puzzletunneldiscovery_gb300 as pw

    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    Ve, Fe, Vr, Fr = _meshes(args.workload)
    uw = pw.UnitWorld(local)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.set_bvh(BVH_KIND)
    uw.angleModel(0.0, 0.0)
    job = RowJob(args.workload, uw, args.n, rank)
    stream = torch.cuda.current_stream(dev)
    # the node boxes of the kernel the workload runs, picked on a sample of its own queries
    from puzzletunneldiscovery_gb300 import sampling as SP
    from puzzletunneldiscovery_gb300.autotune import pick_node_boxes
    if args.workload == "keyconf":
        rp, rn, ep, en = (x[:512] for x in job.pairs)
        hc, hs = _keyconf_half_angles(KEYCONF_SPINS)
        pick_node_boxes(uw, states=SP.keyconf_states(uw, rp, rn, ep, en, KEYCONF_MARGIN, hc, hs).view(-1, 7))
    elif args.workload == "touch":
        pick_node_boxes(uw, segments=SP.touch_segments(uw, job.keys[:256], TOUCH_PER_KEY, 5),
                        verify_delta=uw.recommended_cres)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        res = job.gpu()
    torch.cuda.synchronize(dev)
    step_ms = []
    job.launches = 0
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            if job.device_timed:
                s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s0.record(stream)
                res = job.gpu()
                s1.record(stream)
                torch.cuda.synchronize(dev)
                step_ms.append(s0.elapsed_time(s1))
            else:
                t0 = time.perf_counter()
                res = job.gpu()
                torch.cuda.synchronize(dev)
                step_ms.append(1e3 * (time.perf_counter() - t0))
    ms = sum(step_ms) / len(step_ms)
    value = job.units / (ms / 1e3)
    job.timed_launches = job.launches
    # end to end: host inputs in, host results out, inside the timed region
    if job.device_timed:
        hq = torch.from_numpy(job.q).pin_memory()
        e2e_ms = 0.0
        for i in range(args.steps):
            flush.zero_()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            out = uw.is_disentangled_states(hq.to(dev, non_blocking=True)).cpu()
            s1.record(stream)
            torch.cuda.synchronize(dev)
            e2e_ms += s0.elapsed_time(s1)
        if not torch.equal(out, res.cpu()):
            raise RuntimeError("host-array path disagrees with the device path")
        e2e = {"value": job.units * args.steps / (e2e_ms / 1e3), "unit": job.unit,
               "h2d_bytes_per_step": int(job.q.nbytes), "d2h_bytes_per_step": int(job.n)}
    else:
        # the public call takes host arrays and returns host arrays: the timed steps are end to end
        e2e = {"value": value, "unit": job.unit, "h2d_bytes_per_step": _row_h2d(job),
               "d2h_bytes_per_step": _row_d2h(job, res)}
    if rank != 0:
        return
    roof = None
    if args.workload == "disentangled":
        # one thread per state, FP64 box test: 56 B in, 1 B out per state
        peak, kind = _peaks()
        ach = job.units * 57 / (ms / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": None,
                "kernel": "k_disentangled", "kernel_ms": ms, "peak_source": kind, "algorithmic_bytes": job.units * 57}
    cpu, parity = None, None
    if ws == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        ow = O.OracleWorld(Ve, Fe, Vr, Fr)
        cores = os.cpu_count() or 1
        m = max(1, min(job.n, 64 if args.workload in ("contacts", "keyconf", "touch", "visibility") else 65536))
        while True:
            units, dt, cres = job.cpu(ow, m, cores)
            if dt >= args.cpu_seconds or m >= job.n:
                break
            grow = args.cpu_seconds / max(dt, 1e-3)
            if args.workload == "visibility":
                grow = math.sqrt(grow)               # all pairs among m keys: units grow as m^2
            m = min(job.n, max(m * 2, int(m * grow * 1.05)))
        cpu = {"value": units / dt, "unit": job.unit, "cores": cores, "kind": "port",
               "sample": "the first %d %s of the step (%d units, %.1f s)"
                         % (m, {"disentangled": "states", "contacts": "states", "keyconf": "surface pairs",
                                "touch": "keys", "visibility": "keys (all pairs among them)"}[args.workload], units,
                            dt)}
        parity = {"mismatches": job.mismatches(ow, res, cres, m), "mismatch_sample": int(m),
                  "compared": {"disentangled": "is_disentangled verdict of every state",
                               "contacts": "contact rows (face pairs, segment ends, lengths) of every state",
                               "keyconf": "the free median spins of every surface pair",
                               "touch": "done flag of every segment; full transit tuples of the first 256",
                               "visibility": "every pair's visibility bit among the sampled keys"}[
                      args.workload]}
    cfg = {"workload": "%s/interlocking_tori" % args.workload, "units_per_step": job.units,
           "l2": "flushed (256 MB write) between timed steps",
           "parallelism": "replicas" if ws == 1 else "independent replicas"}
    if args.workload == "keyconf":
        cfg.update({"surface_pairs": job.n, "spins": KEYCONF_SPINS, "margin": KEYCONF_MARGIN, "only_median": True})
    elif args.workload == "touch":
        cfg.update({"keys": job.keys.shape[0], "segments_per_key": TOUCH_PER_KEY, "stepping": uw.recommended_cres})
    elif args.workload == "contacts":
        cfg.update({"states": job.n, "states_drawn_from": "colliding uniform states in [-0.6, 0.6]^3 (world)"})
    elif args.workload == "visibility":
        cfg.update({"keys": job.n, "pairs": job.units, "verify_magnitude": VIS_DELTA,
                    "keys_drawn_from": "free uniform states in [-2, 2]^3 (world)"})
    detail = {"mismatches": parity["mismatches"] if parity else None,
              "mismatch_sample": parity["mismatch_sample"] if parity else 0, "parity": parity, "step_ms": step_ms,
              "node_boxes": {"states": uw.get_node_boxes(0), "segments": uw.get_node_boxes(1)}}
    if args.workload == "contacts":
        detail["contact_rows_per_state"] = float(res[4][-1]) / max(1, job.n)
    if args.workload == "keyconf":
        detail["key_configurations_per_step"] = sum(r.shape[0] for r in res)
    if args.workload == "touch":
        detail["free_fraction"] = float(res[2].mean())
    line = {"metric": WORKLOADS[args.workload][0], "value": value, "unit": job.unit, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 box test" if args.workload == "disentangled" else "f32 traversal + f64 state math/re-tests",
            "data": "synthetic (seeded)", "config": cfg, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clk.summary(),
            # counted by the library per query (CUB's sorts and scans not counted)
            "gpu_launches": job.timed_launches,
            "detail": detail}
    print(json.dumps(line), flush=True)
    if parity and parity["mismatches"]:
        print("verdict mismatches against the oracle: %d" % parity["mismatches"], file=sys.stderr)
        sys.exit(3)


def _row_h2d(job):
    if job.name == "contacts":
        return int(job.q.nbytes)
    if job.name == "visibility":
        return int(job.keys.nbytes)
    if job.name == "keyconf":
        return int(job.n * KEYCONF_SPINS * 56)
    return int(job.units * 2 * 56)


def _row_d2h(job, res):
    if job.name == "visibility":
        return int(job.n * job.n)
    if job.name == "contacts":
        return int(sum(x.nbytes for x in res[:4]) + res[3].shape[0] * 4 + res[4].nbytes)
    if job.name == "keyconf":
        return int(job.n * KEYCONF_SPINS)
    return int(job.units * (2 * 56 + 1 + 8))


class _RefRowJob(RowJob):
    """The row workloads' batches built without a GPU (the oracle answers the
    verdicts the GPU arm uses to pick its colliding or free inputs)."""

    def __init__(self, name, ow, n, Fe, Fr):
        self.name, self.n = name, n
        s = ow.scene_scale
        rng = np.random.default_rng(3000)
        self.uw = type("_Stepping", (), {"recommended_cres": 0.001})()
        if name == "disentangled":
            self.q = W.uniform_states(n, -2.0, 2.0, s, seed=0)
            self.units, self.unit = n, "checks/s"
        elif name == "contacts":
            q = W.uniform_states(8 * n, -0.6, 0.6, s, seed=0)
            self.q = q[~ow.is_valid(q)][:n]
            self.n = self.q.shape[0]
            self.units, self.unit = self.n, "states/s"
        elif name == "visibility":
            q = W.uniform_states(4 * n, -2.0, 2.0, s, seed=0)
            self.keys = np.ascontiguousarray(q[ow.is_valid(q)][:n])
            self.n = self.keys.shape[0]
            self.units, self.unit = self.n * (self.n - 1) // 2, "pairs/s"
        elif name == "keyconf":
            Ve, Vr = ow.vertices(0), ow.vertices(1)
            self.pairs = _surface_pairs(Ve, np.asarray(Fe, np.int64), Vr, np.asarray(Fr, np.int64), n, rng)
            self.units, self.unit = n * KEYCONF_SPINS, "checks/s"
        else:
            from puzzletunneldiscovery_gb300 import sampling as SP
            q = W.uniform_states(4 * n, -2.0, 2.0, s, seed=0)
            self.keys = q[ow.is_valid(q)][:n]
            K = self.keys.shape[0]
            r = np.random.default_rng(4000)
            frm = np.repeat(self.keys, TOUCH_PER_KEY, axis=0)
            self.to = SP.apply_rows(frm, SP.random_on_sphere(K * TOUCH_PER_KEY, 1.0, r),
                                    SP.random_within_sphere(K * TOUCH_PER_KEY, 2 * np.pi, r))
            self.units, self.unit = K * TOUCH_PER_KEY, "segments/s"


def run_rows_reference(args):
    """--impl reference for the row workloads: the oracle on the host cores, a
    bounded sample of the step per timed step."""
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    Ve, Fe, Vr, Fr = _meshes(args.workload)
    ow = O.OracleWorld(Ve, Fe, Vr, Fr)
    job = _RefRowJob(args.workload, ow, args.n, Fe, Fr)
    cores = os.cpu_count() or 1
    per = {"disentangled": 500, "contacts": 1, "keyconf": 1, "touch": 1, "visibility": 1}[args.workload]
    div = {"disentangled": 1, "contacts": 8, "keyconf": 4, "touch": 4, "visibility": 16}[args.workload]
    m = max(1, min(job.n, args.ref_sample // div * per))
    times, units = [], 0
    for it in range(args.warmup + args.steps):
        u, dt, _ = job.cpu(ow, m, cores)
        if it >= args.warmup:
            times.append(dt)
            units += u
    value = units / sum(times)
    line = {"impl": "reference", "metric": WORKLOADS[args.workload][0], "value": value, "unit": job.unit,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, same batch as the GPU arm)",
            "config": {"workload": "%s/interlocking_tori" % args.workload, "units_per_step": job.units,
                       "sample_per_step": m},
            "cpu_baseline": {"value": value, "unit": job.unit, "cores": cores, "kind": "port",
                             "sample": "the first %d of the step's %d inputs per step" % (m, job.n)},
            "e2e": {"value": value, "unit": job.unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["bf16_tflops_sustained"]), "measured (sustained)"
    except Exception:
        return 1700.0, "fallback (sustained)"


def _cpu_plain_sampling(cand, gpu_valid, target_s):
    """Plain uniform sampling on the host cores: the oracle's isValid on the
    first candidates of the GPU's resident batch (grown until it takes about
    target_s), counting the free ones (the reference's sampler has no
    surrogate), and its verdicts compared with the GPU plain arm's.
    Returns (cpu_baseline dict, parity dict)."""
    from oracle import oracle as O
    O.build()
    Ve, Fe, Vr, Fr = _meshes("surrogate")
    ow = O.OracleWorld(Ve, Fe, Vr, Fr)
    cores = os.cpu_count() or 1
    n = 65536
    while True:
        n = min(n, cand.shape[0])
        q = cand[:n].cpu().numpy()
        t0 = time.perf_counter()
        v = ow.is_valid(q, nthreads=cores)
        dt = time.perf_counter() - t0
        if dt >= target_s or n >= min(cand.shape[0], 1 << 26):
            break
        n = max(n * 2, int(n * target_s / max(dt, 1e-3) * 1.1))
    mism = int((v != gpu_valid[:n].astype(bool)).sum())
    cpu = {"value": float(v.sum()) / dt, "unit": "samples/s", "cores": cores, "kind": "port",
           "sample": "first %d uniform candidates of the GPU's batch checked, %d free, %.1f s"
                     % (n, int(v.sum()), dt)}
    parity = {"mismatches": mism, "mismatch_sample": int(n), "compared": "is_valid_state verdict of every candidate",
              "sample": "the CPU-baseline sample, against the plain arm's last timed step"}
    return cpu, parity


def run_surrogate_reference(args):
    """--impl reference for the surrogate workload: plain uniform sampling with the
    CPU restatement of the reference's isValid on all host cores."""
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    Ve, Fe, Vr, Fr = _meshes("surrogate")
    ow = O.OracleWorld(Ve, Fe, Vr, Fr)
    cores = os.cpu_count() or 1
    sample = 200 * args.ref_sample
    times, free = [], 0
    for it in range(args.warmup + args.steps):
        q = W.uniform_states(sample, -2.0, 2.0, ow.scene_scale, seed=500 + it)
        t0 = time.perf_counter()
        v = ow.is_valid(q, nthreads=cores)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
            free += int(v.sum())
    value = free / sum(times)
    line = {"impl": "reference", "metric": WORKLOADS["surrogate"][0], "value": value, "unit": "samples/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform states)",
            "config": {"workload": "surrogate_guided_sampling/interlocking_tori", "candidates_per_step": sample,
                       "method": "plain uniform sampling (the reference has no surrogate)"},
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": "port",
                             "sample": "%d uniform states per step" % sample},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _profile_value(name, key):
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith(key):
                return float(line.split("=")[1])
    except Exception:
        pass
    return None


def _traffic_per_segment():
    """DRAM bytes per segment of the traversal kernel, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_segments_traffic.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_segment"):
                return float(line.split("=")[1])
    except Exception:
        pass
    return None


def run_profile_case(args):
    """Small fixed workloads for ncu captures (no JSON line): `states`, `segments`,
    `mlp`, `train`, `plate`, `ompl`, `disentangled` or `all` (every kernel of the engine once),
    with --n units, on the interlocking tori (the plate and torus knot for
    `plate`, the alpha puzzle for `ompl`); --node-boxes picks the BVH boxes."""
    import torch

    import puzzletunneldiscovery_gb300 as pw
    from puzzletunneldiscovery_gb300 import surrogate as S

    what, n = args.profile_case, args.n
    dev = torch.device("cuda", 0)
    if what == "ompl":
        from puzzletunneldiscovery_gb300 import ompl_compat as OC
        (Ve, Fe, Vr, Fr), c, P = _alpha_ompl()
        uw = pw.UnitWorld(0)
        uw.load_env_mesh(Ve, Fe)
        uw.load_robot_mesh(Vr, Fr)
        uw.enforceRobotCenter(c)
        uw.scaleToUnit()
        uw.set_bvh(BVH_KIND)
        uw.angleModel(0.0, 0.0)
        A, B, lo, hi = _ompl_motions(P, n, 0)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        for _ in range(3):
            v, states = OC._check_motions_dev(uw, a, b, lo, hi, OMPL_CDRES)
        torch.cuda.synchronize()
        print("done", states, float(v.float().mean()))
        return
    Ve, Fe, Vr, Fr = W.cfg_plate_knot() if what == "plate" else W.cfg_interlocking_tori()
    uw = pw.UnitWorld(0)
    uw.load_env_mesh(Ve, Fe)
    uw.load_robot_mesh(Vr, Fr)
    uw.scaleToUnit()
    uw.set_bvh(BVH_KIND)
    uw.angleModel(0.0, 0.0)
    if args.node_boxes:
        uw.set_node_boxes(args.node_boxes)
    s = uw.scene_scale
    if what == "plate":
        q = torch.from_numpy(_batch(n, s, 0, "plate", Ve)[0]).to(dev)
        for _ in range(3):
            uw.is_valid_states(q)
        torch.cuda.synchronize()
        print("done", uw.last_stats())
        return
    if what == "all":
        from puzzletunneldiscovery_gb300 import narrow as N
        q = torch.from_numpy(W.uniform_states(n, -2, 2, s, seed=0)).to(dev)
        uw.is_valid_states(q)
        uw.is_disentangled_states(q)
        q0, q1 = W.segment_batch(max(1, n // 10), -2, 2, s, seed=0)
        a, b = torch.from_numpy(q0).to(dev), torch.from_numpy(q1).to(dev)
        uw.transit_states_to_with_contact(a, b, DELTA)
        uw.intersecting_segments(np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0]))
        uw.intersecting_segments_batch(W.uniform_states(4096, -0.6, 0.6, s, seed=1))
        ends = N.expand(q[:1000], 64, 0.01, 0.1, 5)
        N.crossings(q[:1000], ends, 64, torch.zeros((4, 3), dtype=torch.float64, device=dev), 0.0, 0.5)
        net = S.Surrogate(0, 1)
        sc = net.score(q)
        S.select_top(sc, q, max(1, n // 10))
        net.predict_mma(q[:65536])
        y = uw.is_valid_states(q[:65536])
        net.train_step(q[:65536], y, 1e-3)
        net.set_training_kernels(True)
        net.train_step(q[:65536], y, 1e-3)
        net.check()
        torch.cuda.synchronize()
        print("done")
        return
    if what in ("mlp", "train"):
        net = S.Surrogate(0, 1)
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        q = S.uniform_states_device(n, -2, 2, s, g, dev)
        if what == "mlp":
            for _ in range(3):
                net.predict(q)
            net.check()
        else:
            y = uw.is_valid_states(q[:65536])
            for _ in range(3):
                net.train_step(q[:65536], y, 1e-3)
        torch.cuda.synchronize()
        print("done")
        return
    if what == "disentangled":
        q = torch.from_numpy(W.uniform_states(n, -2, 2, s, seed=0)).to(dev)
        for _ in range(3):
            uw.is_disentangled_states(q)
        torch.cuda.synchronize()
        print("done", uw.last_stats())
        return
    if what == "states":
        q = torch.from_numpy(W.uniform_states(n, -2, 2, s, seed=0)).to(dev)
        for _ in range(3):
            uw.is_valid_states(q)
    else:
        q0, q1 = W.segment_batch(n, -2, 2, s, seed=0)
        a, b = torch.from_numpy(q0).to(dev), torch.from_numpy(q1).to(dev)
        for _ in range(3):
            uw.first_contact_steps(a, b, DELTA)
    torch.cuda.synchronize()
    print("done", uw.last_stats())


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="segments")
    ap.add_argument("--n", type=int, default=None, help="units (segments or states) per GPU")
    ap.add_argument("--ref-sample", type=int, default=2000, help="segments per reference-arm step")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--no-surrogate-arm", action="store_true",
                    help="segments: skip the surrogate-guided sampling figures in the detail")
    ap.add_argument("--narrow-k", type=int, default=65536, help="narrow: segments validated per round")
    ap.add_argument("--narrow-train-labels", type=int, default=10_000_000,
                    help="narrow: exact labels of the initial training")
    ap.add_argument("--train-labels", type=int, default=50_000_000, help="surrogate: exact labels to train on")
    ap.add_argument("--top-frac", type=float, default=0.1, help="surrogate: fraction of candidates checked")
    ap.add_argument("--e2e-n", type=int, default=20_000_000, help="surrogate: candidates per end-to-end step")
    ap.add_argument("--sweep", type=lambda v: [float(x) for x in v.split(",") if x], default=[0.25, 0.5, 0.6],
                    help="surrogate: further checked fractions reported in detail")
    ap.add_argument("--profile-case", choices=["states", "segments", "mlp", "train", "plate", "ompl", "disentangled", "all"],
                    default=None,
                    help="run a small fixed workload for an ncu capture instead of the benchmark")
    ap.add_argument("--bvh", choices=["topdown", "sah", "morton"], default="topdown",
                    help="the BVH hierarchy of the worlds (top-down principal-axis splits or Morton LBVH)")
    ap.add_argument("--node-boxes", choices=["aligned", "oriented"], default=None,
                    help="profile cases: the BVH node boxes (default: the world's default)")
    args = ap.parse_args()
    global BVH_KIND
    BVH_KIND = args.bvh
    if args.profile_case:
        args.n = args.n or 1_000_000
        run_profile_case(args)
        return
    if args.n is None:
        args.n = WORKLOADS[args.workload][2]
    if args.workload == "narrow":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no narrow-passage search with a "
                              "learned proposal; its CPU path is timed in the plate workload"}))
        else:
            run_narrow(args)
    elif args.workload == "ompl":
        run_ompl_reference(args) if args.impl == "reference" else run_ompl(args)
    elif args.workload == "surrogate":
        run_surrogate_reference(args) if args.impl == "reference" else run_surrogate(args)
    elif args.workload in ROW_WORKLOADS:
        run_rows_reference(args) if args.impl == "reference" else run_rows(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
