"""The learned proposal: a BF16 MLP that scores states by P(collision free).

The network and its kernels live in libpwcollide.so (include/pw_mlp.h).  This
module wraps them for PyTorch device tensors and adds the two samplers that
use the scores:

* ``guided_free_samples`` -- rank a batch of candidate states by the network
  and check only the top fraction exactly (pw_states_valid).  Every accepted
  state carries an exact verdict, so the accepted set holds no false-free
  state whatever the network says.
* ``train_online`` -- draw states, label them with the exact kernel, and take
  Adam steps on those labels, all on the device.

The reference has no such component (its learned part, src/hg, predicts
surface heat maps); the samplers feed the same consumers as its key
configuration sampler (src/GP/pipeline/keyconf.py:106-160).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


class Surrogate:
    """One network on one GPU (pw_mlp)."""

    def __init__(self, device: int = 0, seed: int = 0):
        self._L = _lib.load()
        self.device = torch.device("cuda", device)
        h = ctypes.c_void_p()
        _lib.check(self._L.pw_mlp_create(ctypes.byref(h), device, seed), "pw_mlp_create")
        self._h = h
        self.num_params = int(self._L.pw_mlp_num_params(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.pw_mlp_destroy(h)
            self._h = None

    # parameters -------------------------------------------------------------
    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        _lib.check(self._L.pw_mlp_get_params(self._h, out.ctypes.data_as(_lib.fp)), "pw_mlp_get_params")
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.shape != (self.num_params,):
            raise ValueError("expected %d parameters, got %s" % (self.num_params, p.shape))
        _lib.check(self._L.pw_mlp_set_params(self._h, p.ctypes.data_as(_lib.fp)), "pw_mlp_set_params")

    def grads(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        _lib.check(self._L.pw_mlp_get_grads(self._h, out.ctypes.data_as(_lib.fp)), "pw_mlp_get_grads")
        return out

    def adam_state(self) -> dict:
        """Adam's first / second moments (float32 [num_params]) and step count."""
        m1 = np.empty(self.num_params, np.float32)
        m2 = np.empty(self.num_params, np.float32)
        step = ctypes.c_int64()
        _lib.check(self._L.pw_mlp_get_adam(self._h, m1.ctypes.data_as(_lib.fp), m2.ctypes.data_as(_lib.fp),
                                           ctypes.byref(step)), "pw_mlp_get_adam")
        return {"m1": m1, "m2": m2, "step": int(step.value)}

    def set_adam_state(self, state: dict) -> None:
        m1 = np.ascontiguousarray(state["m1"], np.float32)
        m2 = np.ascontiguousarray(state["m2"], np.float32)
        if m1.shape != (self.num_params,) or m2.shape != (self.num_params,):
            raise ValueError("expected Adam moments of %d values" % self.num_params)
        _lib.check(self._L.pw_mlp_set_adam(self._h, m1.ctypes.data_as(_lib.fp), m2.ctypes.data_as(_lib.fp),
                                           int(state["step"])), "pw_mlp_set_adam")

    def state_dict(self) -> dict:
        """Everything a resumed run needs for the same next training step:
        parameters, Adam moments and step count (CPU tensors)."""
        a = self.adam_state()
        return {"format": "pw_mlp/1", "params": torch.from_numpy(self.params()),
                "m1": torch.from_numpy(a["m1"]), "m2": torch.from_numpy(a["m2"]), "step": a["step"]}

    def load_state_dict(self, sd: dict) -> None:
        if sd.get("format") != "pw_mlp/1":
            raise ValueError("not a pw_mlp checkpoint (format %r)" % sd.get("format"))
        self.set_params(sd["params"].numpy())
        self.set_adam_state({"m1": sd["m1"].numpy(), "m2": sd["m2"].numpy(), "step": sd["step"]})

    def save(self, path: str) -> None:
        """Checkpoint with torch.save: parameters and Adam state."""
        torch.save(self.state_dict(), path)

    def load(self, path: str) -> None:
        """Restore a torch.save checkpoint, or a bare float32 parameter array
        saved with numpy (Adam state then left as it is)."""
        if str(path).endswith(".npy"):
            self.set_params(np.load(path))
            return
        self.load_state_dict(torch.load(path, map_location="cpu", weights_only=True))

    # device calls -----------------------------------------------------------
    def _states(self, q):
        if not (isinstance(q, torch.Tensor) and q.is_cuda and q.dtype == torch.float64 and q.dim() == 2
                and q.shape[1] == 7):
            raise TypeError("states must be a CUDA float64 tensor of shape [n, 7]")
        return q.contiguous()

    def predict(self, q: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """P(free) of each state, float32 [n], asynchronous on the current stream."""
        q = self._states(q)
        n = q.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device=q.device)
        _lib.check(self._L.pw_mlp_predict(self._h, ctypes.c_void_p(q.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                          _stream(q.device)), "pw_mlp_predict")
        return out

    def score(self, q: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """The logit of P(free) (no sigmoid), float32 [n]: a ranking score that does not saturate."""
        q = self._states(q)
        n = q.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device=q.device)
        _lib.check(self._L.pw_mlp_score(self._h, ctypes.c_void_p(q.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                        _stream(q.device)), "pw_mlp_score")
        return out

    def predict_mma(self, q: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """The same prediction through the mma.sync GEMM kernels that training uses."""
        q = self._states(q)
        n = q.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.float32, device=q.device)
        _lib.check(self._L.pw_mlp_predict_mma(self._h, ctypes.c_void_p(q.data_ptr()), n,
                                              ctypes.c_void_p(out.data_ptr()), _stream(q.device)),
                   "pw_mlp_predict_mma")
        return out

    def set_training_kernels(self, use_mma: bool) -> None:
        """Train with the mma.sync GEMMs (True) or the tcgen05 GEMMs (False, default)."""
        _lib.check(self._L.pw_mlp_set_training_kernels(self._h, 1 if use_mma else 0), "pw_mlp_set_training_kernels")

    def check(self) -> None:
        """Synchronise; raise if a bounded device wait of an earlier predict gave up."""
        _lib.check(self._L.pw_mlp_check(self._h), "pw_mlp_check")

    def _labels(self, y, n):
        if not (isinstance(y, torch.Tensor) and y.is_cuda and y.shape == (n,)):
            raise TypeError("labels must be a CUDA tensor of shape [n]")
        return y.to(torch.uint8).contiguous()

    def gradients(self, q: torch.Tensor, labels: torch.Tensor) -> float:
        q = self._states(q)
        y = self._labels(labels, q.shape[0])
        loss = ctypes.c_float()
        _lib.check(self._L.pw_mlp_gradients(self._h, ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                            q.shape[0], ctypes.byref(loss), _stream(q.device)), "pw_mlp_gradients")
        return float(loss.value)

    def train_step(self, q: torch.Tensor, labels: torch.Tensor, lr: float = 1e-3, sync_loss: bool = False):
        """One Adam step on a batch; returns the loss when sync_loss (which synchronises)."""
        q = self._states(q)
        y = self._labels(labels, q.shape[0])
        loss = ctypes.c_float()
        _lib.check(self._L.pw_mlp_train_step(self._h, ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                             q.shape[0], float(lr), ctypes.byref(loss) if sync_loss else None,
                                             _stream(q.device)), "pw_mlp_train_step")
        return float(loss.value) if sync_loss else None


# ---------------------------------------------------------------- state draws

def uniform_states_device(n: int, lo: float, hi: float, scale: float, gen: torch.Generator,
                          device) -> torch.Tensor:
    """n states with translation uniform in [lo, hi]^3 (scaled to the unit world by
    `scale`) and a uniform unit quaternion (Shoemake 1992), drawn on the device."""
    u = torch.rand((n, 6), dtype=torch.float64, device=device, generator=gen)
    q = torch.empty((n, 7), dtype=torch.float64, device=device)
    q[:, :3] = (lo + (hi - lo) * u[:, :3]) * scale
    u1, u2, u3 = u[:, 3], u[:, 4] * (2 * math.pi), u[:, 5] * (2 * math.pi)
    a, b = torch.sqrt(1 - u1), torch.sqrt(u1)
    q[:, 3] = a * torch.sin(u2)
    q[:, 4] = a * torch.cos(u2)
    q[:, 5] = b * torch.sin(u3)
    q[:, 6] = b * torch.cos(u3)
    return q


# ---------------------------------------------------------------- training

@dataclass
class TrainReport:
    labels: int = 0
    steps: int = 0
    losses: list = field(default_factory=list)
    free_fraction: float = 0.0


def train_online(world, net: Surrogate, draw, total_labels: int, batch: int = 65536, lr: float = 1e-3,
                 label_chunk: int = 1 << 22, log_every: int = 0) -> TrainReport:
    """Label `total_labels` states from draw(n) with the exact kernel and train on
    them in batches of `batch` (one pass, Adam).  Labels: 1 = collision free."""
    rep = TrainReport()
    free = 0
    while rep.labels < total_labels:
        n = min(label_chunk, total_labels - rep.labels)
        n -= n % batch if n > batch else 0
        q = draw(n)
        y = world.is_valid_states(q)
        free += int(y.sum())
        for s in range(0, n, batch):
            want = log_every and rep.steps % log_every == 0
            loss = net.train_step(q[s:s + batch], y[s:s + batch], lr, sync_loss=bool(want))
            if want:
                rep.losses.append((rep.steps, loss))
            rep.steps += 1
        rep.labels += n
    rep.free_fraction = free / max(rep.labels, 1)
    return rep


# ---------------------------------------------------------------- guided sampling

@dataclass
class GuidedReport:
    candidates: int = 0
    checked: int = 0
    accepted: int = 0
    precision: float = 0.0      # accepted / checked: exact-free among the top fraction


def select_top(score: torch.Tensor, q: torch.Tensor, k: int, slack: int = 1 << 16) -> torch.Tensor:
    """The states whose score is at or above the k-th largest (pw_select_top),
    in no particular order; ties at the threshold are all kept."""
    L = _lib.load()
    if not (isinstance(score, torch.Tensor) and score.dtype == torch.float32 and score.is_cuda
            and score.shape == (q.shape[0],)):
        raise TypeError("score must be a CUDA float32 tensor with one value per state")
    q = q.contiguous()
    cap = min(q.shape[0], k + slack)
    while True:
        out = torch.empty((cap, 7), dtype=torch.float64, device=q.device)
        cnt = ctypes.c_int64()
        rc = L.pw_select_top(ctypes.c_void_p(score.data_ptr()), ctypes.c_void_p(q.data_ptr()), q.shape[0], int(k),
                             ctypes.c_void_p(out.data_ptr()), cap, ctypes.byref(cnt), _stream(q.device))
        if rc == _lib.PW_ERR_CAPACITY:
            cap = int(cnt.value)
            continue
        _lib.check(rc, "pw_select_top")
        return out[:cnt.value]


def guided_free_samples(world, net: Surrogate, q: torch.Tensor, top_frac: float = 0.1, score=None):
    """Rank candidates by the network's logit and check the top `top_frac`
    exactly; returns (accepted free states, GuidedReport).  Every returned
    state passed pw_states_valid."""
    rep = GuidedReport()
    score = net.score(q, out=score)
    k = max(1, int(round(top_frac * q.shape[0])))
    cand = select_top(score, q, k)
    ok = world.is_valid_states(cand)
    acc = cand[ok]
    rep.candidates = int(q.shape[0])
    rep.checked = int(cand.shape[0])
    rep.accepted = int(acc.shape[0])
    rep.precision = rep.accepted / max(rep.checked, 1)
    return acc, rep


def plain_free_samples(world, q: torch.Tensor):
    """Check every candidate exactly; returns the free ones."""
    ok = world.is_valid_states(q)
    return q[ok]


def precision_recall(prob: torch.Tensor, labels: torch.Tensor, threshold: float = 0.5):
    """Precision and recall of `prob >= threshold` as a free-space predictor."""
    pred = prob >= threshold
    y = labels.bool()
    tp = int((pred & y).sum())
    fp = int((pred & ~y).sum())
    fn = int((~pred & y).sum())
    return tp / max(tp + fp, 1), tp / max(tp + fn, 1)
