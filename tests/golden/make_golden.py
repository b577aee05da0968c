"""Generate the golden fixtures in this folder from the Muesli reference itself.

Runs oracle/_ref/ref_harness -- the reference's own OpenMP skeletons (DA/DM/DC
map, zip, index map/zip, fold, DM/DC mapStencil), compiled from the reference
sources by `make -C oracle ref` -- on small seeded inputs and stores inputs and
outputs as <case>.npz. Regenerate with:

    make -C oracle ref && python tests/golden/make_golden.py

Inputs come from numpy's default_rng(seed); the seed of each case is stored in
the fixture. Outputs are the reference's bytes, unchanged.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def run(op, ints, inputs, out_dtype, out_count):
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for k, a in enumerate(inputs):
            p = os.path.join(td, f"in{k}.bin")
            np.ascontiguousarray(a).tofile(p)
            paths.append(p)
        outp = os.path.join(td, "out.bin")
        cmd = [HARNESS, op, *[str(v) for v in ints], "--", *paths, "--", outp]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
        return np.fromfile(outp, dtype=out_dtype, count=out_count)


def jacobi_init(rows, cols, seed):
    """Plain-Jacobi grid: row 0 = 100, other boundary cells 0, inside U[0,1)."""
    g = np.random.default_rng(seed).random((rows, cols), dtype=np.float32)
    g[:, 0] = 0.0
    g[:, -1] = 0.0
    g[-1, :] = 0.0
    g[0, :] = 100.0
    return g


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


def heat3d_special_case():
    """heat3D on values around the GPU division's fast-path range: tiny (1e-38)
    and subnormal (3e-40) cells, +inf cells (never negated, so no sum meets
    inf - inf and no NaN arises), negative cells; a block of zeros holding
    single cells at +-2^-122 x {0.999999, 1, 1.25, 1.4999999, 1.5, 1.5000001,
    2} (a neighbour's first sum is the cell alone) and a block of -0 (the
    reference's sum starts from +0), both through the whole depth and wide
    enough that the other values, one cell per sweep, reach neither the
    single cells nor the -0 block's core within the three sweeps."""
    rng = np.random.default_rng(58)
    c = rng.random((16, 40, 72), dtype=np.float32)  # 288-byte rows: the GPU's TMA kernels take it
    u = rng.random(c.shape)
    c[u < 0.01] = np.float32(1e-38)
    c[(u >= 0.01) & (u < 0.02)] = np.float32(3e-40)
    c[(u >= 0.02) & (u < 0.025)] = np.float32(np.inf)
    c[(u >= 0.025) & (u < 0.05)] *= np.float32(-0.3)
    c[:, 2:22, 2:40] = 0.0
    t = np.float32(2.0 ** -122)
    for k, f in enumerate((1.0, 1.25, 1.4999999, 1.5, 1.5000001, 2.0, 0.999999)):
        c[5 + (k % 2) * 4, 6 + 2 * k, 6 + 5 * k] = np.float32(f) * t * np.float32(1 if k % 2 else -1)
    c[:, 24:38, 44:62] = np.float32(-0.0)
    ints = [16, 40, 72, 3]
    save("dc_heat3d_special", seed=58, ints=ints, in0=c, out=run("dc_heat3d", ints, [c], np.float32, c.size))


def main():
    if not os.path.exists(HARNESS):
        sys.exit(f"missing {HARNESS}: run `make -C oracle ref` first")
    rng = np.random.default_rng

    # DA<float> map / zip / fold (the float part of the map/zip/fold microbench).
    n = 4099
    x = rng(42).uniform(-1, 1, n).astype(np.float32)
    y = rng(43).uniform(-1, 1, n).astype(np.float32)
    for op in ("da_map_affine", "da_map_inplace_affine"):
        save(op, seed=42, ints=[n], in0=x, out=run(op, [n], [x], np.float32, n))
    for op in ("da_zip_muladd", "da_zip_inplace_muladd"):
        save(op, seed=[42, 43], ints=[n], in0=x, in1=y, out=run(op, [n], [x, y], np.float32, n))
    for op in ("da_fold_sum_f32", "da_fold_max_f32"):
        save(op, seed=42, ints=[n], in0=x, out=run(op, [n], [x], np.float32, 1))

    # DA<int> part: mapIndex x ^ (i & 1023), fold(+) with int32 wrap-around.
    xi = rng(44).integers(0, 1000, n, dtype=np.int32)
    save("da_mapindex_xor", seed=44, ints=[n], in0=xi, out=run("da_mapindex_xor", [n], [xi], np.int32, n))
    save("da_fold_sum_i32", seed=44, ints=[n], in0=xi, out=run("da_fold_sum_i32", [n], [xi], np.int32, 1))
    big = rng(45).integers(0, 2**30, 64, dtype=np.int32)  # sum wraps past 2^31
    save("da_fold_sum_i32_wrap", seed=45, ints=[64], in0=big, out=run("da_fold_sum_i32", [64], [big], np.int32, 1))

    # Index skeletons with non-commutative functors (pin the argument order).
    a = rng(46).integers(-500, 500, n, dtype=np.int32)
    b = rng(47).integers(-500, 500, n, dtype=np.int32)
    save("da_mapindex_inplace", seed=46, ints=[n], in0=a, out=run("da_mapindex_inplace", [n], [a], np.int32, n))
    for op in ("da_zipindex", "da_zipindex_inplace"):
        save(op, seed=[46, 47], ints=[n], in0=a, in1=b, out=run(op, [n], [a, b], np.int32, n))
    rows, cols = 37, 53
    a2 = rng(48).integers(-500, 500, (rows, cols), dtype=np.int32)
    b2 = rng(49).integers(-500, 500, (rows, cols), dtype=np.int32)
    for op in ("dm_mapindex", "dm_mapindex_inplace"):
        save(op, seed=48, ints=[rows, cols], in0=a2, out=run(op, [rows, cols], [a2], np.int32, rows * cols))
    for op in ("dm_zipindex", "dm_zipindex_inplace"):
        save(op, seed=[48, 49], ints=[rows, cols], in0=a2, in1=b2,
             out=run(op, [rows, cols], [a2, b2], np.int32, rows * cols))
    d3 = (5, 7, 11)
    a3 = rng(50).integers(-500, 500, d3, dtype=np.int32)
    b3 = rng(51).integers(-500, 500, d3, dtype=np.int32)
    n3 = int(np.prod(d3))
    for op in ("dc_mapindex", "dc_mapindex_inplace"):
        save(op, seed=50, ints=list(d3), in0=a3, out=run(op, list(d3), [a3], np.int32, n3))
    for op in ("dc_zipindex", "dc_zipindex_inplace"):
        save(op, seed=[50, 51], ints=list(d3), in0=a3, in1=b3, out=run(op, list(d3), [a3, b3], np.int32, n3))

    # DM::mapStencil: plain Jacobi (fixed boundary), heat2D with a non-zero
    # neutral value, Game of Life, box mean over the radius sweep.
    g = jacobi_init(48, 64, 42)
    save("dm_jacobi5", seed=42, ints=[48, 64, 10], in0=g, out=run("dm_jacobi5", [48, 64, 10], [g], np.float32, g.size))
    res = run("dm_jacobi_residual", [48, 64, 100], [g], np.float32, g.size + 1)
    save("dm_jacobi_residual", seed=42, ints=[48, 64, 100], in0=g, out=res[:-1], residual=res[-1:])
    h = rng(52).random((33, 47), dtype=np.float32)
    save("dm_heat2d", seed=52, ints=[33, 47, 3, 500], in0=h,
         out=run("dm_heat2d", [33, 47, 3, 500], [h], np.float32, h.size))
    life = (rng(53).random((64, 80)) < 0.3).astype(np.int32)
    save("dm_life8", seed=53, ints=[64, 80, 20], in0=life, out=run("dm_life8", [64, 80, 20], [life], np.int32, life.size))
    blur = rng(54).uniform(0, 255, (40, 56)).astype(np.float32)
    for r in (1, 2, 4, 6, 8, 10):
        save(f"dm_boxmean_r{r}", seed=54, ints=[40, 56, r, 1], in0=blur,
             out=run("dm_boxmean", [40, 56, r, 1], [blur], np.float32, blur.size))
    small = rng(55).uniform(0, 255, (13, 17)).astype(np.float32)  # radius larger than half the grid
    save("dm_boxmean_r10_small", seed=55, ints=[13, 17, 10, 2], in0=small,
         out=run("dm_boxmean", [13, 17, 10, 2], [small], np.float32, small.size))

    # DC::mapStencil: heat3D, Dirichlet 0 outside; 3-D box sums (meanblur).
    c = rng(56).random((12, 10, 14), dtype=np.float32)
    save("dc_heat3d", seed=56, ints=[12, 10, 14, 5], in0=c, out=run("dc_heat3d", [12, 10, 14, 5], [c], np.float32, c.size))
    heat3d_special_case()
    cb = rng(57).random((9, 10, 11), dtype=np.float32)
    for r in (1, 2):
        save(f"dc_boxsum_r{r}", seed=57, ints=[9, 10, 11, r, 1], in0=cb,
             out=run("dc_boxsum", [9, 10, 11, r, 1], [cb], np.float32, cb.size))
    # DM row / column skeletons: reduceRows (int sum with wrap-around; max over
    # positive floats, where the CPU build's 0 seed is neutral), reducetwoColumns,
    # rotateRows / rotateCols (both signs, |a| >= size), setColumn.
    ri = rng(58).integers(-2**30, 2**30, (41, 77), dtype=np.int32)
    save("dm_reduce_rows_sum_i32", seed=58, ints=[41, 77], in0=ri,
         out=run("dm_reduce_rows_sum_i32", [41, 77], [ri], np.int32, 41))
    wide = rng(59).integers(-1000, 1000, (5, 2500), dtype=np.int32)
    save("dm_reduce_rows_sum_i32_wide", seed=59, ints=[5, 2500], in0=wide,
         out=run("dm_reduce_rows_sum_i32", [5, 2500], [wide], np.int32, 5))
    rf = rng(60).random((41, 77), dtype=np.float32)
    save("dm_reduce_rows_max_f32", seed=60, ints=[41, 77], in0=rf,
         out=run("dm_reduce_rows_max_f32", [41, 77], [rf], np.float32, 41))
    tc = rng(61).uniform(-1, 1, (23, 19)).astype(np.float32)
    save("dm_reduce_two_columns", seed=61, ints=[23, 19], in0=tc,
         out=run("dm_reduce_two_columns", [23, 19], [tc], np.float32, 23))
    rot = rng(62).integers(-1000, 1000, (11, 13), dtype=np.int32)
    for tag, a in (("p2", 2), ("m3", -3), ("p11", 11), ("p12", 12)):
        save(f"dm_rotate_rows_{tag}", seed=62, ints=[11, 13, a], in0=rot,
             out=run("dm_rotate_rows", [11, 13, a], [rot], np.int32, rot.size))
    for tag, a in (("p3", 3), ("m5", -5), ("m30", -30), ("p13", 13)):
        save(f"dm_rotate_cols_{tag}", seed=62, ints=[11, 13, a], in0=rot,
             out=run("dm_rotate_cols", [11, 13, a], [rot], np.int32, rot.size))
    sc = rng(63).random((17, 9), dtype=np.float32)
    sv = rng(64).random(17, dtype=np.float32)
    save("dm_set_column", seed=[63, 64], ints=[17, 9, 4], in0=sc, in1=sv,
         out=run("dm_set_column", [17, 9, 4], [sc, sv], np.float32, sc.size))

    # DM x DA broadcast zips and the DA-with-matrix-rows skeletons (int32,
    # non-commutative functors of oracle/ref_harness.cpp).
    for tag, (rows, cols) in (("7x5", (7, 5)), ("33x40", (33, 40)), ("16x16", (16, 16))):
        g = rng(65 + rows)
        a = g.integers(-1000, 1000, (rows, cols), dtype=np.int32)
        b = g.integers(-1000, 1000, (rows, cols), dtype=np.int32)
        u, v, w = (g.integers(-1000, 1000, rows, dtype=np.int32) for _ in range(3))
        ops = ["dm_zipindex_ma", "dm_zipindex_a", "dm_zipindex_aaa"] + (["dm_crosszip"] if rows == cols else [])
        for op in ops:
            save(f"{op}_{tag}", seed=65 + rows, ints=[rows, cols], in0=a, in1=b, in2=u, in3=v, in4=w,
                 out=run(op, [rows, cols], [a, b, u, v, w], np.int32, a.size))
        for op in ("da_mapindex_dmrows", "da_zipindex_dmrows"):
            save(f"{op}_{tag}", seed=65 + rows, ints=[rows, cols], in0=a, in1=u, in2=v,
                 out=run(op, [rows, cols], [a, u, v], np.int32, rows))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
