"""Learned step-size proposer for the DOP853 integrator.

An 8 -> 64 -> 64 -> 1 ReLU MLP with BF16 weights and FP32 accumulation,
trained and evaluated on the tensor cores by the library's own kernels
(csrc/mlp.cuh, csrc/mlp_train.cu, csrc/learned.cu).  Inputs: the particle's
lon, lat, model time, velocity (u, v) and velocity gradient (du/dx, du/dy,
dv/dx) at the start of a step; output: log of the step the dop853 controller
would have chosen had it known the step's error, log(|h| 0.9 err^(-1/8)).

Training data come from the integrator itself (:func:`log_steps`); at run
time ``flowmap_grid_2D(..., precision="mixed", step_model=proposer)`` lets the
network propose each step while the embedded error estimate still accepts or
rejects it, so the plain controller remains the fallback and the arbiter.
"""
import ctypes

import numpy as np
import torch

from . import _device as D
from . import _lib
from .flows import _check_callable_flow

N_IN, N_HID = 8, 64
FEATURES = ("lon", "lat", "t", "u", "v", "du_dx", "du_dy", "dv_dx")


def log_steps(flow, t0, T, x, y, params, rtol=1e-6, atol=1e-8, sample=1.0, seed=0,
              capacity=1 << 22):
    """Integrate the grid with the plain controller (mixed precision) and
    return (features (n, 8), targets (n,)) float32 CUDA tensors for a hashed
    fraction ``sample`` of the accepted steps that start and end inside the
    velocity grid (at most ``capacity`` rows) and the number of samples
    offered."""
    D.require_cuda()
    flow = _check_callable_flow(flow)
    xd, yd = D.to_dev(x), D.to_dev(y)
    prm = np.ascontiguousarray(params, dtype=np.float64)
    feats = D.empty((capacity, N_IN), torch.float32)
    targ = D.empty((capacity,), torch.float32)
    count = torch.zeros(1, dtype=torch.int64, device=D.device())
    L = _lib.load()
    _lib.check(L.nbcs_flowmap_log_steps(flow.struct, float(t0), float(T), D.ptr(xd), xd.numel(),
                                        D.ptr(yd), yd.numel(), prm.ctypes.data_as(_lib._vp),
                                        len(prm), float(rtol), float(atol), float(sample),
                                        int(seed) & 0xFFFFFFFF, D.ptr(feats), D.ptr(targ),
                                        capacity, D.ptr(count), D.stream_ptr()))
    n = int(count.item())
    k = min(n, capacity)
    return feats[:k], targ[:k], n


class StepProposer:
    """MLP weights (FP32 master copy + BF16 device blob) and their training."""

    def __init__(self, seed=0):
        D.require_cuda()
        L = _lib.load()
        self.nparam = L.nbcs_mlp_param_count()
        rng = np.random.default_rng(seed)
        p = np.zeros(self.nparam, np.float32)
        # Kaiming-uniform for the ReLU layers, small output layer
        p[0:512] = rng.uniform(-1, 1, 512) * np.sqrt(6.0 / N_IN)
        p[576:4672] = rng.uniform(-1, 1, 4096) * np.sqrt(6.0 / N_HID)
        p[4736:4800] = rng.uniform(-1, 1, 64) * np.sqrt(1.0 / N_HID)
        self.params = torch.from_numpy(p).to(D.device())
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.loss_buf = torch.zeros(1, dtype=torch.float32, device=D.device())
        nb = L.nbcs_mlp_blob_bytes()
        self.blob = torch.zeros((nb + 15) // 16 * 16, dtype=torch.uint8, device=D.device())
        self.norm = np.zeros(20, np.float32)  # mu[8], inv_sigma[8], out_mu, out_sigma, (b3, pad)
        self.norm[8:16] = 1.0
        self.norm[17] = 1.0
        self.step = 0
        self.margin = 0.0  # log of the proposal margin (see proposal_blob)
        self._version = 0
        self._proposal = None
        self._write_norm()
        self._pack()

    # -- blob maintenance
    def _write_norm(self):
        hdr = self.blob[:72].view(torch.float32)
        hdr[:18] = torch.from_numpy(self.norm[:18]).to(D.device())
        self._version += 1

    def _pack(self):
        _lib.check(_lib.load().nbcs_mlp_pack(D.ptr(self.params), D.ptr(self.blob), D.stream_ptr()))
        self._version += 1

    def proposal_blob(self):
        """The blob the integrator proposes steps with: the trained network
        with its log-step output shifted by ``margin``.  The network predicts
        the ideal step with a log-space error of about one standard
        deviation, and min(proposal, controller) picks that error's low tail;
        a margin > 0 lets the proposal cut only steps it is confident are too
        long.  ``margin`` is calibrated on training flows (bench.py)."""
        key = (self._version, float(self.margin))
        if self._proposal is None or self._proposal[0] != key:
            b = self.blob.clone()
            hdr = b[:72].view(torch.float32)
            hdr[16] = float(self.norm[16]) + float(self.margin)
            self._proposal = (key, b)
        return self._proposal[1]

    def set_normalization(self, feats, targets):
        f = feats.double()
        mu = f.mean(0)
        sd = f.std(0).clamp_min(1e-12)
        self.norm[0:8] = mu.float().cpu().numpy()
        self.norm[8:16] = (1.0 / sd).float().cpu().numpy()
        t = targets.double()
        self.norm[16] = float(t.mean())
        self.norm[17] = float(t.std().clamp_min(1e-12))
        self._write_norm()

    @property
    def consts(self):
        return self.norm[0:8], self.norm[8:16], float(self.norm[16]), float(self.norm[17])

    # -- compute
    def gradient(self, feats, targets):
        """(grad tensor (nparam,), mean squared error in standardised units)."""
        f, t = feats.contiguous(), targets.contiguous()
        _lib.check(_lib.load().nbcs_mlp_grad(D.ptr(self.blob), D.ptr(f), D.ptr(t), t.numel(),
                                             D.ptr(self.grad), D.ptr(self.loss_buf),
                                             D.stream_ptr()))
        return self.grad, float(self.loss_buf.item()) / max(1, t.numel())

    def predict(self, feats):
        f = feats.contiguous()
        out = D.empty((f.shape[0],), torch.float32)
        _lib.check(_lib.load().nbcs_mlp_predict(D.ptr(self.blob), D.ptr(f), f.shape[0], D.ptr(out),
                                                D.stream_ptr()))
        return out

    def mse(self, feats, targets):
        """Mean squared error in standardised target units."""
        p = self.predict(feats)
        return float((((p - targets) / self.norm[17]) ** 2).mean())

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        _lib.check(_lib.load().nbcs_mlp_adam(D.ptr(self.params), D.ptr(self.m), D.ptr(self.v),
                                             D.ptr(self.grad), ctypes.c_float(lr),
                                             ctypes.c_float(beta1), ctypes.c_float(beta2),
                                             ctypes.c_float(eps), self.step, D.ptr(self.blob),
                                             D.stream_ptr()))
        self._version += 1

    def train(self, feats, targets, epochs=4, batch=65536, lr=3e-3, lr_final=3e-4, seed=0,
              val=None, log=None):
        """Adam on mini-batches (reshuffled each epoch), cosine-decayed rate.
        Returns the per-epoch history of training (and validation) MSE."""
        n = targets.numel()
        if self.step == 0:
            self.set_normalization(feats, targets)
        g = torch.Generator(device=feats.device).manual_seed(seed)
        steps = epochs * ((n + batch - 1) // batch)
        hist = []
        k = 0
        for ep in range(epochs):
            perm = torch.randperm(n, generator=g, device=feats.device)
            tot = 0.0
            for s in range(0, n, batch):
                idx = perm[s:s + batch]
                frac = k / max(1, steps - 1)
                rate = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * frac))
                _, l = self.gradient(feats.index_select(0, idx), targets.index_select(0, idx))
                self.adam_step(rate)
                tot += l * idx.numel()
                k += 1
            rec = {"epoch": ep, "train_mse": tot / n}
            if val is not None:
                rec["val_mse"] = self.mse(*val)
            hist.append(rec)
            if log:
                log(rec)
        return hist

    def save(self, path):
        np.savez(path, params=self.params.cpu().numpy(), norm=self.norm, step=self.step,
                 margin=self.margin)

    @classmethod
    def load(cls, path):
        z = np.load(path)
        sp = cls()
        sp.params.copy_(torch.from_numpy(z["params"]).to(sp.params.device))
        sp.norm = z["norm"].astype(np.float32)
        sp.step = int(z["step"])
        sp.margin = float(z["margin"]) if "margin" in z.files else 0.0
        sp._write_norm()
        sp._pack()
        return sp
