"""The learned warm start: a BF16 U-Net trained and run by the library's own
CUDA kernels (libpcd_gb300: pcd_unet_*).

    net = UNet(ctx, resolution=256, max_batch=16, seed=0)
    x, t = make_pairs(ctx, seeds, 256)          # right-hand sides and solved potentials
    train(net, x, t, epochs=..., batch=16)
    net.attach(ctx)                             # solves with warm_start=2 use it
    net.save("unet256.npz")

The network maps x = (b - mean b) / std(b) to phi_hat = phi / (std(b) * S^2)
(mean removed); a solve on an N x N grid resamples b to S x S, predicts, and
uses phi0 = N^2 * std(b_S) * bilinear(phi_hat) as its initial guess, kept only
if its residual is below ||b||.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib, inputs
from ._lib import check
from .solver import STOP_REL_RESIDUAL, Context, SolveOptions, batch_solve

# (Cin, Cout, level) of the 14 3x3 convolutions, in parameter order; then the
# 1x1 head (32 weights, 1 bias).  Weights of a convolution are [Cout][Kp] with
# k = tap * Cin + ci (tap = 3*ky + kx), Kp = 9*Cin rounded up to 32.
LAYERS = [(1, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 128, 2), (128, 128, 2), (128, 256, 3),
          (256, 256, 3), (384, 128, 2), (128, 128, 2), (192, 64, 1), (64, 64, 1), (96, 32, 0), (32, 32, 0)]


def _round32(k):
    return (k + 31) // 32 * 32


def param_layout():
    """[(name, offset, shape)] of the flat FP32 parameter vector."""
    out, off = [], 0
    for i, (ci, co, _) in enumerate(LAYERS):
        kp = _round32(9 * ci)
        out.append((f"conv{i}.w", off, (co, kp)))
        off += co * kp
        out.append((f"conv{i}.b", off, (co,)))
        off += co
    out.append(("head.w", off, (32,)))
    off += 32
    out.append(("head.b", off, (1,)))
    off += 1
    return out, off


class UNet:
    def __init__(self, ctx: Context, resolution: int = 256, max_batch: int = 16, seed: int = 0):
        self._L = _lib.load()
        self.ctx = ctx
        h = C.c_void_p()
        check(self._L.pcd_unet_create(ctx.handle, int(resolution), int(max_batch), int(seed), C.byref(h)),
              "pcd_unet_create")
        self._h = h
        self.resolution = resolution
        self.max_batch = max_batch
        self.n = int(self._L.pcd_unet_num_params(h))

    def close(self):
        if self._h:
            self._L.pcd_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        check(self._L.pcd_unet_get_params(self._h, out.ctypes.data), "pcd_unet_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n
        check(self._L.pcd_unet_set_params(self._h, p.ctypes.data), "pcd_unet_set_params")

    def grads(self) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        check(self._L.pcd_unet_get_grads(self._h, out.ctypes.data), "pcd_unet_get_grads")
        return out

    def save(self, path: str, half: bool = False):
        """Writes the parameters (float16 with ``half``: the network computes
        in BF16, whose 8-bit significand float16's 11 bits cover)."""
        p = self.get_params()
        np.savez_compressed(path, params=p.astype(np.float16) if half else p, resolution=self.resolution)

    def load(self, path: str):
        z = np.load(path)
        if int(z["resolution"]) != self.resolution:
            raise ValueError("weights were trained at another resolution")
        self.set_params(np.asarray(z["params"], dtype=np.float32))

    def train_step(self, x, target, lr: float, weight_decay: float = 0.0) -> float:
        """x, target: CUDA float32 tensors [B, S, S]."""
        import torch

        B = x.shape[0]
        loss = C.c_float(0)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        check(self._L.pcd_unet_train_step(self._h, x.data_ptr(), target.data_ptr(), B, float(lr), float(weight_decay),
                                          C.byref(loss), C.c_void_p(stream)), "pcd_unet_train_step")
        return loss.value

    def predict(self, x):
        import torch

        out = torch.empty_like(x)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        check(self._L.pcd_unet_predict(self._h, x.data_ptr(), x.shape[0], out.data_ptr(), C.c_void_p(stream)),
              "pcd_unet_predict")
        return out

    def attach(self, ctx: Context | None = None):
        check(self._L.pcd_ctx_set_warm_start_net((ctx or self.ctx).handle, self._h), "pcd_ctx_set_warm_start_net")


def make_pairs(ctx: Context, seeds, S: int = 256, tol: float = 1e-7, chunk: int = 256, net_res: int | None = None):
    """Right-hand sides b (Gaussian mixtures for even seeds, binary shapes for
    odd ones) on S x S grids and their potentials, solved on the GPU by the
    batched solver.  With net_res < S both are area-averaged to net_res x
    net_res (the grid the network runs on; the library averages a solve's b
    the same way before inference).  Returns CUDA float32 tensors x (the
    averaged b) and target = averaged phi / (std(x) * S^2), the scaling the
    library inverts with the std of its averaged input and the solve grid's
    W * H."""
    import torch
    import torch.nn.functional as F

    R = net_res or S
    if S % R:
        raise ValueError("the data grid must be a multiple of the network grid")
    xs, ts = [], []
    opts = SolveOptions(stop=STOP_REL_RESIDUAL, tol=tol, max_iterations=200000, omega=-1.0, warm_start=0)
    seeds = list(seeds)
    for i in range(0, len(seeds), chunk):
        part = seeds[i:i + chunk]
        bb = inputs.poisson_rhs_torch(S, part)
        bs = [bb[k] for k in range(len(part))]
        phis = [torch.zeros_like(b) for b in bs]
        batch_solve(ctx, bs, phis, opts)
        for b, p in zip(bs, phis):
            if R != S:
                b = F.avg_pool2d(b[None, None], S // R)[0, 0]
                p = F.avg_pool2d(p[None, None], S // R)[0, 0]
            sd = b.std()
            xs.append(b.float())
            ts.append((p / (sd * S * S)).float())
    return torch.stack(xs), torch.stack(ts)


def train(net: UNet, x, t, epochs: int = 4, batch: int = 16, lr: float = 2e-3, weight_decay: float = 1e-5,
          seed: int = 0, log=None, time_budget_s: float | None = None):
    """AdamW with a cosine learning-rate decay; returns the per-epoch mean loss.

    With ``time_budget_s`` the step count is cut, after the first 50 steps
    have been timed, to what fits the budget (the cosine schedule is rescaled
    to the shorter run)."""
    import time

    import torch

    g = torch.Generator(device="cpu").manual_seed(seed)
    n = x.shape[0]
    steps = epochs * (n // batch)
    k, hist = 0, []
    t0 = time.time()
    for ep in range(epochs):
        if k >= steps:
            break
        perm = torch.randperm(n, generator=g).to(x.device)
        tot, cnt = 0.0, 0
        for i in range(0, n - batch + 1, batch):
            if k >= steps:
                break
            if time_budget_s is not None and k == 50:
                per = (time.time() - t0) / k
                steps = min(steps, max(51, int(time_budget_s / per)))
            idx = perm[i:i + batch]
            lr_k = lr * 0.5 * (1 + np.cos(np.pi * k / max(1, steps)))
            loss = net.train_step(x[idx].contiguous(), t[idx].contiguous(), lr_k, weight_decay)
            tot += loss
            cnt += 1
            k += 1
        hist.append(tot / max(1, cnt))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4e}")
    return hist


def default_weights_path(resolution: int = 64) -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", f"unet{resolution}.npz")
