"""Seeded synthetic inputs with the shapes and value distributions of the
caustic-design workloads (no image files are read).

* ``gaussian_image``: the 8-bit target image of the full-pipeline workload --
  sum of isotropic Gaussians (centres U[0.1,0.9]^2, sigma U[0.03,0.15],
  amplitude U[0.2,1]) over a 0.05 floor, normalised to max 255, quantised.
* ``gray_from_u8``: the gray value the reference's PNG loader produces for an
  R=G=B pixel (main.cpp:91-99).
* ``resize_nearest``: main.cpp:13-27.
* ``density``: target densities for the single and batched Poisson solves --
  16-Gaussian mixtures or binary shapes (20 disks/rectangles at 1 on a 0.02
  floor), normalised to mean 1.
* ``poisson_rhs``: b = density - 1 with the mean removed exactly in FP64.
"""
from __future__ import annotations

import numpy as np


def _gaussians(n_w: int, n_h: int, rng, k: int) -> np.ndarray:
    y, x = np.meshgrid((np.arange(n_h) + 0.5) / n_h, (np.arange(n_w) + 0.5) / n_w, indexing="ij")
    img = np.zeros((n_h, n_w))
    for _ in range(k):
        cx, cy = rng.uniform(0.1, 0.9, size=2)
        s = rng.uniform(0.03, 0.15)
        a = rng.uniform(0.2, 1.0)
        img += a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
    return img


def gaussian_image(n: int = 128, seed: int = 0, k: int = 8, floor: float = 0.05) -> np.ndarray:
    """uint8 (n, n) target image."""
    rng = np.random.default_rng(seed)
    img = floor + _gaussians(n, n, rng, k)
    return np.round(img / img.max() * 255.0).astype(np.uint8)


def gray_from_u8(img: np.ndarray) -> np.ndarray:
    """Gray value of an R=G=B 8-bit pixel as main.cpp:91-99 computes it."""
    r = img.astype(np.float64) / 255.0
    return (0.299 * r) + (0.587 * r) + (0.114 * r)


def resize_nearest(img: np.ndarray, new_w: int, new_h: int) -> np.ndarray:
    """Nearest-neighbour resize with integer source indices (main.cpp:13-27)."""
    old_h, old_w = img.shape
    ys = (np.arange(new_h) * old_h) // new_h
    xs = (np.arange(new_w) * old_w) // new_w
    return np.ascontiguousarray(img[ys][:, xs])


def pipeline_image(mesh_res: int, seed: int = 0, image_n: int = 128) -> np.ndarray:
    """Gray grid fed to Caustic_design.initialize_solvers for a square target:
    a seeded image_n^2 8-bit image resized to (4*mesh_res)^2 (main.cpp:216-222)."""
    g = gray_from_u8(gaussian_image(image_n, seed))
    return resize_nearest(g, 4 * mesh_res, 4 * mesh_res)


def density(n: int, seed: int = 0, kind: str = "gaussian", m: int | None = None) -> np.ndarray:
    """Mean-1 target density on an (m or n) x n grid."""
    rng = np.random.default_rng(seed)
    h = n if m is None else m
    if kind == "gaussian":
        rho = 0.05 + _gaussians(n, h, rng, 16)
    elif kind == "binary":
        y, x = np.meshgrid((np.arange(h) + 0.5) / h, (np.arange(n) + 0.5) / n, indexing="ij")
        rho = np.full((h, n), 0.02)
        for _ in range(20):
            cx, cy = rng.uniform(0.05, 0.95, size=2)
            if rng.uniform() < 0.5:
                r = rng.uniform(0.03, 0.15)
                rho[(x - cx) ** 2 + (y - cy) ** 2 <= r * r] = 1.0
            else:
                hw, hh = rng.uniform(0.03, 0.15, size=2)
                rho[(np.abs(x - cx) <= hw) & (np.abs(y - cy) <= hh)] = 1.0
    else:
        raise ValueError(f"unknown density kind {kind!r}")
    return rho / rho.mean()


def poisson_rhs(n: int, seed: int = 0, kind: str = "gaussian", m: int | None = None) -> np.ndarray:
    """b = rho - 1, mean removed exactly (two-pass FP64)."""
    b = density(n, seed, kind, m) - 1.0
    b -= b.mean()
    b -= b.mean()
    return np.ascontiguousarray(b)


def poisson_rhs_torch(n: int, seeds, device="cuda"):
    """Batched GPU version of ``poisson_rhs`` for training data: for each seed
    the same parameters are drawn (Gaussian mixture for even seeds, binary
    shapes for odd seeds) and the fields are evaluated with torch in FP64.
    Returns an [len(seeds), n, n] float64 tensor of mean-free right-hand sides."""
    import torch

    y = (torch.arange(n, device=device, dtype=torch.float64) + 0.5) / n
    Y, X = torch.meshgrid(y, y, indexing="ij")
    out = []
    for s in seeds:
        rng = np.random.default_rng(s)
        if s % 2 == 0:
            rho = torch.full((n, n), 0.05, device=device, dtype=torch.float64)
            for _ in range(16):
                cx, cy = rng.uniform(0.1, 0.9, size=2)
                sg = rng.uniform(0.03, 0.15)
                a = rng.uniform(0.2, 1.0)
                rho += a * torch.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * sg * sg))
        else:
            rho = torch.full((n, n), 0.02, device=device, dtype=torch.float64)
            for _ in range(20):
                cx, cy = rng.uniform(0.05, 0.95, size=2)
                if rng.uniform() < 0.5:
                    r = rng.uniform(0.03, 0.15)
                    rho[(X - cx) ** 2 + (Y - cy) ** 2 <= r * r] = 1.0
                else:
                    hw, hh = rng.uniform(0.03, 0.15, size=2)
                    rho[((X - cx).abs() <= hw) & ((Y - cy).abs() <= hh)] = 1.0
        b = rho / rho.mean() - 1.0
        b = b - b.mean()
        b = b - b.mean()
        out.append(b)
    return torch.stack(out)
