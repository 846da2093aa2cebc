"""Launch-shape autotuner and CUDA-graph replay for the traversal kernels.

``pick_bvh`` rebuilds a world with each BVH hierarchy (top-down principal-axis
splits, or the Morton LBVH) and keeps the faster one with its faster node-box
kind for a sample of the caller's queries.  ``autotune`` times the persistent
traversal kernels of one world on a sample of the caller's own workload: first
the two kinds of BVH node box (axis-aligned or
oriented, pw_world_set_node_boxes, per kernel), then, under the faster one, a grid of
launch configurations (queries a warp takes per grab, traversal stack soft cap
-- the point where a warp narrows from breadth-first to depth-first -- and
resident blocks per SM).  Every choice must return the same verdicts; the
fastest is kept (pw_world_set_launch_config).  The best configuration depends on the meshes
(BVH depth, how often queries collide), so it is chosen per world and can be
cached per (mesh pair, GPU model) in a JSON file (``TuneCache``).

``SegmentGraph`` captures one ``pw_segments_first_contact`` call over a
resident batch into a CUDA graph (graph mode: no host synchronisation, no
allocation) and replays it: the whole batch -- bounds, scan, set-up, sort,
rounds, the persistent traversal, FP64 re-tests, finalisation -- is one graph
launch.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
import tempfile
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib


def _time(fn, reps, stream):
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best, out


@dataclass
class TuneReport:
    kernel: str
    best: dict
    default_ms: float
    best_ms: float
    table: list = field(default_factory=list)     # (config, ms)


def _tune_boxes(uw, kernel, run, reps, stream, what):
    """Time `run` under both node-box kinds of `kernel` (default launch shape) and
    keep the faster kind; the two must give identical results.  Returns (kind,
    {kind: ms}, the results)."""
    times, outs = {}, {}
    for kind in ("aligned", "oriented"):
        uw.set_node_boxes(kind, kernel)
        run()
        times[kind], outs[kind] = _time(run, reps, stream)
    if not torch.equal(outs["aligned"], outs["oriented"]):
        raise RuntimeError("the node-box kinds gave different %s" % what)
    kind = min(times, key=times.get)
    uw.set_node_boxes(kind, kernel)
    return kind, times, outs[kind]


def pick_node_boxes(uw, states: torch.Tensor | None = None, segments=None, verify_delta: float = 0.001,
                    mode: int = _lib.PW_SEG_TRANSIT, reps: int = 1) -> dict:
    """Only the node-box kind of each kernel given a sample (states [N, 7], or
    segments (q0, q1) stepped at verify_delta in `mode`): both kinds timed, the
    faster kept.  Returns {"states": kind, "segments": kind, "ms": {...}} for the
    kernels sampled."""
    out = {"ms": {}}
    if states is not None:
        stream = torch.cuda.current_stream(states.device)
        out["states"], out["ms"]["states"], _ = _tune_boxes(uw, 0, lambda: uw.is_valid_states(states), reps, stream,
                                                             "verdicts")
    if segments is not None:
        q0, q1 = segments
        stream = torch.cuda.current_stream(q0.device)
        run = lambda: uw.first_contact_steps(q0, q1, verify_delta, mode)  # noqa: E731
        out["segments"], out["ms"]["segments"], _ = _tune_boxes(uw, 1, run, reps, stream, "first-contact steps")
    return out


def pick_bvh(uw, states: torch.Tensor | None = None, segments=None, verify_delta: float = 0.001,
             mode: int = _lib.PW_SEG_TRANSIT, reps: int = 1, run=None, kernel: int | None = None) -> dict:
    """The BVH hierarchy and node-box kind for a world's workload: the world is
    rebuilt with each hierarchy (pw_world_set_bvh, then angleModel), the box
    kinds timed under each on the sample (states [N, 7], segments (q0, q1), or
    any callable `run` returning a tensor, with the traversal `kernel` it
    exercises: 0 states, 1 segments), and the fastest pair kept (the world is
    left built with it).  Every combination must give the same results.
    Returns {"bvh": kind, "boxes": {...}, "ms": {hierarchy: {box kind: ms}}}."""
    if sum(x is not None for x in (states, segments, run)) != 1:
        raise ValueError("pick_bvh: give one of states, segments or run")
    if run is not None:
        if kernel not in (0, 1):
            raise ValueError("pick_bvh: a run needs its kernel (0 states, 1 segments)")
        what = "results"
        dev = torch.device("cuda", torch.cuda.current_device())
    elif states is not None:
        kernel, dev, what = 0, states.device, "verdicts"
        run = lambda: uw.is_valid_states(states)  # noqa: E731
    else:
        kernel, dev, what = 1, segments[0].device, "first-contact steps"
        run = lambda: uw.first_contact_steps(segments[0], segments[1], verify_delta, mode)  # noqa: E731
    stream = torch.cuda.current_stream(dev)
    ms, ref, best = {}, None, None
    for bvh in ("topdown", "morton"):
        uw.set_bvh(bvh)
        uw.angleModel(0.0, 0.0)
        kind, times, out = _tune_boxes(uw, kernel, run, reps, stream, what)
        if ref is None:
            ref = out
        elif not torch.equal(ref, out):
            raise RuntimeError("the BVH hierarchies gave different %s" % what)
        ms[bvh] = times
        if best is None or times[kind] < best[2]:
            best = (bvh, kind, times[kind])
    if uw.get_bvh() != best[0]:
        uw.set_bvh(best[0])
        uw.angleModel(0.0, 0.0)
    uw.set_node_boxes(best[1], kernel)
    return {"bvh": best[0], "boxes": {"states" if kernel == 0 else "segments": best[1]}, "ms": ms}


def tune_states(uw, q: torch.Tensor, widths=(8, 16, 32), soft_caps=(128, 256, 512, 0), blocks=(0, 2, 3),
                reps: int = 2) -> TuneReport:
    """Pick the states-kernel configuration that answers `q` fastest: first the
    node-box kind, then the launch shape under it."""
    stream = torch.cuda.current_stream(q.device)
    uw.set_launch_config(0)
    kind, box_ms, ref = _tune_boxes(uw, 0, lambda: uw.is_valid_states(q), reps, stream, "verdicts")
    default_ms = box_ms[kind]
    table = []
    for w, c, b in itertools.product(widths, soft_caps, blocks):
        uw.set_launch_config(0, w, c, b)
        uw.is_valid_states(q)
        ms, out = _time(lambda: uw.is_valid_states(q), reps, stream)
        if not torch.equal(out, ref):
            raise RuntimeError("launch configuration %s changed verdicts" % ((w, c, b),))
        table.append(({"width": w, "soft_cap": c, "blocks": b}, ms))
    cfg, ms = min(table, key=lambda t: t[1])
    if ms < default_ms:
        uw.set_launch_config(0, cfg["width"], cfg["soft_cap"], cfg["blocks"])
    else:
        cfg, ms = {"width": 0, "soft_cap": 0, "blocks": 0}, default_ms
        uw.set_launch_config(0)
    cfg = dict(cfg, boxes=kind)
    return TuneReport("states", cfg, default_ms, ms, table + [({"boxes": k}, v) for k, v in box_ms.items()])


def tune_segments(uw, q0: torch.Tensor, q1: torch.Tensor, verify_delta: float, soft_caps=(128, 256, 512, 0),
                  blocks=(0, 2, 3), reps: int = 2, mode: int = _lib.PW_SEG_TRANSIT) -> TuneReport:
    """Pick the segments-kernel configuration that answers (q0, q1) fastest: first
    the node-box kind, then the launch shape under it."""
    stream = torch.cuda.current_stream(q0.device)
    uw.set_launch_config(1)
    run = lambda: uw.first_contact_steps(q0, q1, verify_delta, mode)  # noqa: E731
    kind, box_ms, ref = _tune_boxes(uw, 1, run, reps, stream, "first-contact steps")
    default_ms = box_ms[kind]
    table = []
    for c, b in itertools.product(soft_caps, blocks):
        uw.set_launch_config(1, 0, c, b)
        run()
        ms, out = _time(run, reps, stream)
        if not torch.equal(out, ref):
            raise RuntimeError("launch configuration %s changed first-contact steps" % ((c, b),))
        table.append(({"soft_cap": c, "blocks": b}, ms))
    cfg, ms = min(table, key=lambda t: t[1])
    if ms < default_ms:
        uw.set_launch_config(1, 0, cfg["soft_cap"], cfg["blocks"])
    else:
        cfg, ms = {"soft_cap": 0, "blocks": 0}, default_ms
        uw.set_launch_config(1)
    cfg = dict(cfg, boxes=kind)
    return TuneReport("segments", cfg, default_ms, ms, table + [({"boxes": k}, v) for k, v in box_ms.items()])


def tune_key(meshes, device_name: str, num_sms: int, kernel: str, extra: str = "") -> str:
    """Cache key of a tuned configuration: the mesh pair's arrays (env and robot
    vertices and faces as loaded), the GPU model and SM count, and the kernel."""
    h = hashlib.sha256()
    for m in meshes:
        if m is None:
            h.update(b"none")
            continue
        for a in m:
            a = np.ascontiguousarray(a)
            h.update(str((a.dtype.str, a.shape)).encode())
            h.update(a.tobytes())
    h.update(("%s|%d|%s|%s" % (device_name, num_sms, kernel, extra)).encode())
    return h.hexdigest()


class TuneCache:
    """Tuned configurations per (mesh pair, GPU), in a JSON file.  The default
    file is $PW_AUTOTUNE_CACHE, else ~/.cache/puzzletunneldiscovery_gb300/autotune.json.
    Writes go through a temporary file and a rename, so a reader never sees a
    partial file; two processes writing at once keep the last writer's entries."""

    def __init__(self, path: str | None = None):
        self.path = path or os.environ.get("PW_AUTOTUNE_CACHE") or os.path.join(
            os.path.expanduser("~"), ".cache", "puzzletunneldiscovery_gb300", "autotune.json")

    def load(self) -> dict:
        try:
            with open(self.path) as fh:
                d = json.load(fh)
            return d if isinstance(d, dict) else {}
        except (OSError, ValueError):
            return {}

    def get(self, key: str):
        return self.load().get(key)

    def put(self, key: str, value: dict) -> None:
        d = self.load()
        d[key] = value
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=os.path.dirname(os.path.abspath(self.path)), suffix=".tmp")
        with os.fdopen(fd, "w") as fh:
            json.dump(d, fh, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def _world_key(uw, kernel: str) -> str:
    props = torch.cuda.get_device_properties(uw._device)
    return tune_key(uw._meshes, props.name, props.multi_processor_count, kernel, "%.17g" % uw.scene_scale)


def _apply(uw, kernel: str, cfg: dict) -> None:
    if "boxes" in cfg:
        uw.set_node_boxes(cfg["boxes"], 0 if kernel == "states" else 1)
    if kernel == "states":
        uw.set_launch_config(0, cfg.get("width", 0), cfg.get("soft_cap", 0), cfg.get("blocks", 0))
    else:
        uw.set_launch_config(1, 0, cfg.get("soft_cap", 0), cfg.get("blocks", 0))


def autotune(uw, states: torch.Tensor | None = None, segments=None, verify_delta: float = 0.001,
             cache: "TuneCache | str | bool | None" = None, **kw):
    """Tune both kernels on samples of the caller's workload; returns the reports.

    Each kernel gets its own node-box kind (axis-aligned or oriented BVH boxes)
    and launch shape.

    With a cache (True for the default file, a path, or a TuneCache) a
    configuration already tuned for the same mesh pair on the same GPU model is
    applied without timing anything (its report has an empty table); a new one
    is stored after tuning."""
    tc = None
    if cache is True:
        tc = TuneCache()
    elif isinstance(cache, str):
        tc = TuneCache(cache)
    elif isinstance(cache, TuneCache):
        tc = cache
    out = {}
    jobs = []
    if states is not None:
        jobs.append(("states", lambda: tune_states(uw, states, **kw)))
    if segments is not None:
        jobs.append(("segments", lambda: tune_segments(uw, segments[0], segments[1], verify_delta, **kw)))
    for kernel, run in jobs:
        key = _world_key(uw, kernel) if tc is not None else None
        hit = tc.get(key) if tc is not None else None
        if hit is not None:
            _apply(uw, kernel, hit["config"])
            out[kernel] = TuneReport(kernel, dict(hit["config"]), float(hit["default_ms"]), float(hit["best_ms"]))
            continue
        r = run()
        if tc is not None:
            tc.put(key, {"config": r.best, "default_ms": r.default_ms, "best_ms": r.best_ms,
                         "configs_tried": len(r.table)})
        out[kernel] = r
    return out


class SegmentGraph:
    """pw_segments_first_contact over a resident batch, captured into a CUDA graph.

    The batch first runs normally (sizing the world's scratch), then the world
    switches to graph mode and one call is captured.  ``replay()`` re-runs the
    whole query as one graph launch on the current stream and returns the
    output tensor (overwritten in place).  Inputs must stay at the same
    addresses; their contents may change if the scratch still fits (otherwise
    the affected segments report PW_STEP_INVALID and ``errors()`` is non-zero).

    The graph holds the addresses of the world's scratch buffers.  Any query
    made on the same world outside graph mode may grow (move) them, so every
    replay first compares the world's scratch epoch with the one captured and
    captures again when it changed.
    """

    def __init__(self, uw, q0: torch.Tensor, q1: torch.Tensor, verify_delta: float, mode: int = _lib.PW_SEG_TRANSIT):
        self.uw = uw
        self.q0, self.q1 = uw._dev_states(q0), uw._dev_states(q1)
        self.delta, self.mode = float(verify_delta), int(mode)
        self.captures = 0
        self._capture()

    def _capture(self):
        uw = self.uw
        dev = self.q0.device
        uw.first_contact_steps(self.q0, self.q1, self.delta, self.mode)      # sizes the scratch
        torch.cuda.synchronize(dev)
        uw.set_graph_mode(True)
        self.graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        try:
            with torch.cuda.stream(side):
                with torch.cuda.graph(self.graph, stream=side):
                    self.out = uw.first_contact_steps(self.q0, self.q1, self.delta, self.mode)
        finally:
            uw.set_graph_mode(False)
        torch.cuda.current_stream(dev).wait_stream(side)
        self.epoch = uw.scratch_epoch()
        self.captures += 1

    def replay(self) -> torch.Tensor:
        if self.uw.scratch_epoch() != self.epoch:
            self._capture()
        self.graph.replay()
        return self.out

    def errors(self) -> int:
        torch.cuda.synchronize(self.q0.device)
        return int(self.uw.last_stats().get("device_errors", 0))
