"""Surrogate-guided narrow-passage search: escapes of a robot through the holes
of a plate.

Free roots are expanded into perturbed endpoints (Gaussian translation,
Gaussian rotation vector applied on the left, as osr::apply does).  A
geometric filter (``pw_expansion_crossings``) keeps the expansions along
which some point of the robot's centre line crosses the plate plane inside
the plate; a collision-free such motion passes the robot through a hole.  The
proposal network scores the endpoints of those candidates, the top k of each
round are validated exactly as segments (``pw_segments_first_contact`` in
is_valid_transition mode, replayed as one CUDA graph), and the free ones are
the escapes.  Endpoint labels of the validated candidates feed the network,
which is retrained every ``retrain_labels`` labels.  The plain search
validates k random candidates instead.

An escape is only ever counted after the exact segment query found the
motion free, so the set of escapes holds no false-free motion whatever the
network scores.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .autotune import SegmentGraph
from .surrogate import Surrogate, uniform_states_device


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def centre_line_probes(uw, rings: int, ring_size: int, every: int = 8) -> np.ndarray:
    """Points of a tube robot's centre line in its local unit frame: the means of
    every `every`-th ring of `ring_size` vertices (vertex i * ring_size + j)."""
    V, _ = uw._cd(1)
    V = V[: rings * ring_size].reshape(rings, ring_size, 3)
    return V[::every].mean(axis=1)


def expand(roots: torch.Tensor, per_root: int, sigma_t: float, sigma_rot: float, seed: int) -> torch.Tensor:
    """per_root endpoints per root (pw_expand_states): t + N(0, sigma_t^2 I), and the
    rotation by a rotation vector ~ N(0, sigma_rot^2 I) applied on the left
    (osr_state.cc:244-259).  The same seed gives the same endpoints."""
    L = _lib.load()
    roots = roots.contiguous()
    out = torch.empty((roots.shape[0] * per_root, 7), dtype=torch.float64, device=roots.device)
    _lib.check(L.pw_expand_states(ctypes.c_void_p(roots.data_ptr()), roots.shape[0], int(per_root),
                                  float(sigma_t), float(sigma_rot), ctypes.c_uint64(seed & (2**64 - 1)),
                                  ctypes.c_void_p(out.data_ptr()), _stream(roots.device)), "pw_expand_states")
    return out


def crossings(roots, ends, per_root: int, probes: torch.Tensor, plane_z: float, extent: float) -> torch.Tensor:
    L = _lib.load()
    out = torch.empty(ends.shape[0], dtype=torch.uint8, device=ends.device)
    _lib.check(L.pw_expansion_crossings(ctypes.c_void_p(roots.data_ptr()), ctypes.c_void_p(ends.data_ptr()),
                                        ends.shape[0], int(per_root), ctypes.c_void_p(probes.data_ptr()),
                                        probes.shape[0], float(plane_z), float(extent),
                                        ctypes.c_void_p(out.data_ptr()), _stream(ends.device)),
               "pw_expansion_crossings")
    return out.bool()


def midpoints(frm: torch.Tensor, to: torch.Tensor) -> torch.Tensor:
    """interpolate(frm, to, 1/2): the translation average and the slerp midpoint,
    which is the normalised sum of the two unit quaternions (sign-aligned)."""
    out = torch.empty_like(to)
    out[:, :3] = 0.5 * (frm[:, :3] + to[:, :3])
    qa = frm[:, 3:] / torch.linalg.vector_norm(frm[:, 3:], dim=1, keepdim=True)
    qb = to[:, 3:] / torch.linalg.vector_norm(to[:, 3:], dim=1, keepdim=True)
    sgn = torch.where((qa * qb).sum(dim=1, keepdim=True) < 0, -1.0, 1.0)
    m = qa + sgn * qb
    out[:, 3:] = m / torch.linalg.vector_norm(m, dim=1, keepdim=True)
    return out


def draw_free_roots(uw, n: int, lo, hi, gen: torch.Generator, chunk: int = 1 << 22) -> torch.Tensor:
    """n collision-free states, translation uniform in the box [lo, hi] (world
    units, scaled to the unit frame), uniform rotation."""
    dev = uw._device
    got, total = [], 0
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    while total < n:
        q = uniform_states_device(chunk, 0.0, 1.0, 1.0, gen, dev)
        q[:, :3] = (torch.from_numpy(lo).to(dev) + q[:, :3] * torch.from_numpy(hi - lo).to(dev)) * uw.scene_scale
        q = q[uw.is_valid_states(q)]
        got.append(q)
        total += q.shape[0]
    return torch.cat(got)[:n].contiguous()


@dataclass
class SearchReport:
    rounds: int = 0
    candidates: int = 0
    crossing: int = 0
    validated: int = 0
    escapes: int = 0
    labels: int = 0
    retrains: int = 0
    seconds: float = 0.0
    escape_states: list = field(default_factory=list)   # (from, to) device tensors of the escapes
    validated_states: tuple | None = None   # (from, to, codes) of the first round's validated motions

    @property
    def escapes_per_s(self):
        return self.escapes / self.seconds if self.seconds > 0 else 0.0

    @property
    def yield_(self):
        return self.escapes / max(1, self.validated)


class NarrowPassageSearch:
    """One world (plate + robot), one network; rounds of expansion, filter,
    ranking and exact validation."""

    def __init__(self, uw, net: Surrogate | None, probes: np.ndarray, plane_z: float, extent: float,
                 per_root: int = 64, sigma_t: float = 0.05, sigma_rot: float = 0.1, k: int = 65536,
                 verify_delta: float = 0.001, retrain_labels: int = 10_000_000, seed: int = 0):
        self.uw, self.net = uw, net
        self.dev = uw._device
        self.probes = torch.from_numpy(np.ascontiguousarray(probes, np.float64)).to(self.dev)
        self.plane_z, self.extent = float(plane_z), float(extent)
        self.per_root, self.k = int(per_root), int(k)
        self.sigma_t = float(sigma_t) * uw.scene_scale      # world units -> unit frame
        self.sigma_rot = float(sigma_rot)
        self.delta = float(verify_delta)
        self.retrain_labels = int(retrain_labels)
        self.gen = torch.Generator(device=self.dev)
        self.gen.manual_seed(seed)
        self.seed, self.calls = int(seed), 0
        self._lab_q, self._lab_y, self._nlab = [], [], 0
        # static segment buffers, validated by one captured graph per round
        self.a = torch.zeros((self.k, 7), dtype=torch.float64, device=self.dev)
        self.b = torch.zeros((self.k, 7), dtype=torch.float64, device=self.dev)
        self.a[:, 3] = 1.0
        self.b[:, 3] = 1.0
        self.graph = None

    def _next_seed(self) -> int:
        self.calls += 1
        return (self.seed * 0x9E3779B97F4A7C15 + self.calls) & (2**64 - 1)

    def state_dict(self, include_network: bool = True) -> dict:
        """Search progress as seeded counters: the expansion seed and call count
        (a round's endpoints are a pure function of the two), the generator
        state behind the shuffles and the plain arm's picks, the labels waiting
        for the next retraining (CPU copies), and the network with its Adam
        state.  Taken between rounds; a search restored from it draws the same
        next round."""
        sd = {"format": "pw_narrow/1", "seed": self.seed, "calls": self.calls,
              "gen": self.gen.get_state(),
              "pending_q": [q.cpu() for q in self._lab_q], "pending_y": [y.cpu() for y in self._lab_y]}
        if include_network and self.net is not None:
            sd["net"] = self.net.state_dict()
        return sd

    def load_state_dict(self, sd: dict) -> None:
        if sd.get("format") != "pw_narrow/1":
            raise ValueError("not a narrow-passage search checkpoint (format %r)" % sd.get("format"))
        self.seed, self.calls = int(sd["seed"]), int(sd["calls"])
        self.gen.set_state(sd["gen"])
        self._lab_q = [q.to(self.dev) for q in sd["pending_q"]]
        self._lab_y = [y.to(self.dev) for y in sd["pending_y"]]
        self._nlab = sum(int(q.shape[0]) for q in self._lab_q)
        if "net" in sd:
            if self.net is None:
                raise ValueError("checkpoint holds a network but this search has none")
            self.net.load_state_dict(sd["net"])

    def _validate(self, frm, to):
        """First-contact codes (is_valid_transition mode) of up to k segments via the graph."""
        m = frm.shape[0]
        self.a[:m].copy_(frm)
        self.b[:m].copy_(to)
        if m < self.k:
            self.a[m:].copy_(self.a[:1].expand(self.k - m, 7))   # zero-length fillers: no step is checked
            self.b[m:].copy_(self.a[:1].expand(self.k - m, 7))
        if self.graph is None:
            # size the scratch for this batch with headroom, so that later batches of the
            # same distribution replay without a new capture
            self._reserve(1.5)
            self.graph = SegmentGraph(self.uw, self.a, self.b, self.delta, _lib.PW_SEG_TRANSITION)
        out = self.graph.replay()
        if bool((out == _lib.PW_STEP_INVALID).any()):
            # longer segments than the reserved scratch holds: reserve more and capture again
            self._reserve(2.0)
            self.graph._capture()
            out = self.graph.replay()
        return out[:m]

    def _reserve(self, headroom: float):
        """Reserve segment scratch for the current k buffers times `headroom`: chunk
        counts bounded from the distances (translation norm + rotation angle,
        the engine's metric) of the segments in the buffers."""
        qa = self.a[:, 3:] / torch.linalg.vector_norm(self.a[:, 3:], dim=1, keepdim=True)
        qb = self.b[:, 3:] / torch.linalg.vector_norm(self.b[:, 3:], dim=1, keepdim=True)
        ang = 2.0 * torch.acos(torch.clamp((qa * qb).sum(dim=1).abs(), max=1.0))
        dist = torch.linalg.vector_norm(self.b[:, :3] - self.a[:, :3], dim=1) + ang
        # is_valid_transition steps at min(dist / 2, delta): at least 2 steps per segment
        chunks = torch.ceil((torch.ceil(dist / self.delta) + 2.0) / 32.0) + 1.0
        total = int(chunks.sum().item() * headroom) + 1024
        longest = int(chunks.max().item() * headroom) + 8
        self.uw.segments_reserve(self.k, total, longest)

    def _label(self, q, y):
        if self.net is None:
            return 0
        self._lab_q.append(q)
        self._lab_y.append(y.to(torch.uint8))
        self._nlab += q.shape[0]
        if self._nlab < self.retrain_labels:
            return 0
        Q, Y = torch.cat(self._lab_q), torch.cat(self._lab_y)
        perm = torch.randperm(Q.shape[0], device=self.dev, generator=self.gen)
        for s in range(0, Q.shape[0] - 65535, 65536):
            idx = perm[s:s + 65536]
            self.net.train_step(Q[idx], Y[idx], 1e-3)
        self._lab_q, self._lab_y, self._nlab = [], [], 0
        return 1

    def pretrain(self, roots: torch.Tensor, labels: int, roots_per_round: int = 1 << 20, batch: int = 65536,
                 lr: float = 1e-3) -> int:
        """Train the network on exact labels of the midpoints and endpoints of the
        crossing expansions of `roots` (the search's own candidate distribution);
        returns the number of Adam steps."""
        steps, seen = 0, 0
        while seen < labels:
            for r0 in range(0, roots.shape[0], roots_per_round):
                R = roots[r0:r0 + roots_per_round]
                ends = expand(R, self.per_root, self.sigma_t, self.sigma_rot, self._next_seed())
                idx = torch.nonzero(crossings(R, ends, self.per_root, self.probes, self.plane_z,
                                              self.extent)).flatten()
                if idx.shape[0] == 0:
                    continue
                ct = ends.index_select(0, idx)
                q = torch.cat([midpoints(R.index_select(0, idx // self.per_root), ct), ct])
                y = self.uw.is_valid_states(q)
                perm = torch.randperm(q.shape[0], device=self.dev, generator=self.gen)
                for s in range(0, q.shape[0] - batch + 1, batch):
                    sel = perm[s:s + batch]
                    self.net.train_step(q[sel], y[sel], lr)
                    steps += 1
                seen += q.shape[0]
                if seen >= labels:
                    break
        return steps

    def run(self, roots: torch.Tensor, guided: bool, roots_per_round: int = 1 << 20,
            keep_escapes: bool = False, keep_validated: bool = False) -> SearchReport:
        rep = SearchReport()
        torch.cuda.synchronize(self.dev)
        t0 = time.perf_counter()
        for r0 in range(0, roots.shape[0], roots_per_round):
            R = roots[r0:r0 + roots_per_round]
            ends = expand(R, self.per_root, self.sigma_t, self.sigma_rot, self._next_seed())
            cross = crossings(R, ends, self.per_root, self.probes, self.plane_z, self.extent)
            idx = torch.nonzero(cross).flatten()
            rep.candidates += ends.shape[0]
            rep.crossing += int(idx.shape[0])
            if idx.shape[0] == 0:
                rep.rounds += 1
                continue
            k = min(self.k, int(idx.shape[0]))
            if guided and self.net is not None:
                # a crossing motion is free only if the robot threads the hole: score the
                # motion's midpoint and its endpoint, and rank by the weaker of the two
                cf = R.index_select(0, idx // self.per_root)
                ct = ends.index_select(0, idx)
                score = torch.minimum(self.net.score(midpoints(cf, ct)), self.net.score(ct))
                pick = idx[torch.topk(score, k, sorted=False).indices]
            else:
                pick = idx[torch.randperm(idx.shape[0], device=self.dev, generator=self.gen)[:k]]
            frm = R.index_select(0, pick // self.per_root)
            to = ends.index_select(0, pick)
            codes = self._validate(frm, to)
            free = codes == _lib.PW_STEP_FREE
            rep.validated += k
            rep.escapes += int(free.sum())
            if keep_escapes:
                rep.escape_states.append((frm[free].clone(), to[free].clone()))
            if keep_validated and rep.validated_states is None:
                rep.validated_states = (frm.clone(), to.clone(), codes.clone())
            # exact labels of the validated motions' midpoints train the network
            if guided and self.net is not None:
                mid = midpoints(frm, to)
                rep.retrains += self._label(mid, self.uw.is_valid_states(mid))
                rep.labels += k
            rep.rounds += 1
        torch.cuda.synchronize(self.dev)
        rep.seconds = time.perf_counter() - t0
        return rep
