"""Seeded synthetic inputs of the benchmark workloads (numpy, host memory).

The reference's examples draw inputs from unseeded rand(); these generators
give the same shapes and value distributions from numpy's default_rng(seed),
so the GPU path and the CPU oracle see identical bits.
"""
from __future__ import annotations

import numpy as np


def uniform_f32(n: int, lo: float, hi: float, seed: int) -> np.ndarray:
    """U[lo, hi) float32 (the map/zip/fold microbench inputs)."""
    g = np.random.default_rng(seed)
    out = np.empty(n, np.float32)
    step = 1 << 24
    for s in range(0, n, step):
        e = min(n, s + step)
        out[s:e] = g.uniform(lo, hi, e - s).astype(np.float32)
    return out


def uniform_i32(n: int, lo: int, hi: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).integers(lo, hi, n, dtype=np.int32)


def jacobi_grid(rows: int, cols: int, seed: int = 42) -> np.ndarray:
    """Plain-Jacobi grid: row 0 = 100, the other boundary cells 0, inside U[0,1)."""
    g = np.random.default_rng(seed).random((rows, cols), dtype=np.float32)
    g[:, 0] = 0.0
    g[:, -1] = 0.0
    g[-1, :] = 0.0
    g[0, :] = 100.0
    return g


def blur_image(rows: int, cols: int, seed: int = 42) -> np.ndarray:
    """Mean-blur input: U[0, 255] float32."""
    return np.random.default_rng(seed).uniform(0.0, 255.0, (rows, cols)).astype(np.float32)


def life_board(rows: int, cols: int, seed: int = 42, p: float = 0.3) -> np.ndarray:
    """Game of Life board: Bernoulli(p) live cells as int32 0/1."""
    return (np.random.default_rng(seed).random((rows, cols), dtype=np.float32) < p).astype(np.int32)


def heat_cube(depth: int, rows: int, cols: int, seed: int = 42) -> np.ndarray:
    """Heat-diffusion cube: U[0,1) inside (Dirichlet 0 outside via the neutral value)."""
    g = np.random.default_rng(seed)
    out = np.empty((depth, rows, cols), np.float32)
    for z in range(depth):
        out[z] = g.random((rows, cols), dtype=np.float32)
    return out
