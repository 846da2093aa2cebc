"""Launch-shape autotuner and CUDA-graph replay for the traversal kernels.

``autotune`` times the persistent traversal kernels of one world over a grid of
launch configurations (queries a warp takes per grab, traversal stack soft cap
-- the point where a warp narrows from breadth-first to depth-first -- and
resident blocks per SM) on a sample of the caller's own workload, checks that
every configuration returns the same verdicts, and keeps the fastest
(pw_world_set_launch_config).  The best configuration depends on the meshes
(BVH depth, how often queries collide), so it is chosen per world.

``SegmentGraph`` captures one ``pw_segments_first_contact`` call over a
resident batch into a CUDA graph (graph mode: no host synchronisation, no
allocation) and replays it: the whole batch -- bounds, scan, set-up, sort,
rounds, the persistent traversal, FP64 re-tests, finalisation -- is one graph
launch.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

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


def tune_states(uw, q: torch.Tensor, widths=(8, 16, 32), soft_caps=(128, 256, 512, 0), blocks=(0, 2, 3),
                reps: int = 2) -> TuneReport:
    """Pick the states-kernel configuration that answers `q` fastest."""
    stream = torch.cuda.current_stream(q.device)
    uw.set_launch_config(0)
    uw.is_valid_states(q)
    default_ms, ref = _time(lambda: uw.is_valid_states(q), reps, stream)
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
    return TuneReport("states", cfg, default_ms, ms, table)


def tune_segments(uw, q0: torch.Tensor, q1: torch.Tensor, verify_delta: float, soft_caps=(128, 256, 512, 0),
                  blocks=(0, 2, 3), reps: int = 2, mode: int = _lib.PW_SEG_TRANSIT) -> TuneReport:
    """Pick the segments-kernel configuration that answers (q0, q1) fastest."""
    stream = torch.cuda.current_stream(q0.device)
    uw.set_launch_config(1)
    run = lambda: uw.first_contact_steps(q0, q1, verify_delta, mode)  # noqa: E731
    run()
    default_ms, ref = _time(run, reps, stream)
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
    return TuneReport("segments", cfg, default_ms, ms, table)


def autotune(uw, states: torch.Tensor | None = None, segments=None, verify_delta: float = 0.001, **kw):
    """Tune both kernels on samples of the caller's workload; returns the reports."""
    out = {}
    if states is not None:
        out["states"] = tune_states(uw, states, **kw)
    if segments is not None:
        out["segments"] = tune_segments(uw, segments[0], segments[1], verify_delta, **kw)
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
