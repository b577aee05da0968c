"""The bit-sliced Life update used by life_bits_kernel, restated with numpy on
32-cell words, against the oracle's cell-by-cell Life (the reference's rule,
examples/gameoflife.cpp:22-42): the neighbour words by funnel shifts, the
counts by full adders, the rule `c1 & ~c2 & (c0 | alive)`. No GPU involved:
this checks the algebra the kernel relies on, for every neighbourhood and on
whole boards with the dead border."""
import itertools

import numpy as np

from muesli4_gb300 import abi as A
from oracle import pyoracle as O

M32 = np.uint64(0xFFFFFFFF)


def xor3(a, b, c):
    return a ^ b ^ c


def maj3(a, b, c):
    return (a & b) | (c & (a | b))


def rule_bits(alive, nbrs):
    """The kernel's count-and-rule logic for eight neighbour bit-vectors."""
    lv_a, a, rv_a, lv_b, rv_b, lv_c, c, rv_c = nbrs
    fs_a, fc_a = xor3(lv_a, a, rv_a), maj3(lv_a, a, rv_a)
    fs_c, fc_c = xor3(lv_c, c, rv_c), maj3(lv_c, c, rv_c)
    hs, hc = lv_b ^ rv_b, lv_b & rv_b
    c0, k1 = xor3(fs_a, hs, fs_c), maj3(fs_a, hs, fs_c)
    t, u = xor3(fc_a, hc, fc_c), maj3(fc_a, hc, fc_c)
    c1, c2 = t ^ k1, u ^ (t & k1)
    return c1 & ~c2 & (c0 | alive)


def test_every_neighbourhood():
    for bits in itertools.product([0, 1], repeat=9):
        alive, nb = bits[0], bits[1:]
        s = sum(nb)
        want = 1 if (alive == 1 and s in (2, 3)) or (alive == 0 and s == 3) else 0
        got = rule_bits(alive, list(nb)) & 1
        assert got == want, (alive, nb)


def pack(board):
    """rows x cols 0/1 -> rows x ceil(cols/32) words, bit i = cell 32w + i."""
    rows, cols = board.shape
    nw = (cols + 31) // 32
    padded = np.zeros((rows, nw * 32), np.uint64)
    padded[:, :cols] = board
    weights = (np.uint64(1) << np.arange(32, dtype=np.uint64))
    return (padded.reshape(rows, nw, 32) * weights).sum(axis=2).astype(np.uint64)


def unpack(words, cols):
    rows, nw = words.shape
    bits = (words[:, :, None] >> np.arange(32, dtype=np.uint64)) & np.uint64(1)
    return bits.reshape(rows, nw * 32)[:, :cols].astype(np.int32)


def generation(words, cols):
    rows, nw = words.shape
    z = np.zeros((1, nw), np.uint64)
    up = np.vstack([z, words[:-1]])     # row above (dead border)
    down = np.vstack([words[1:], z])    # row below

    def shifts(w):
        prev = np.hstack([np.zeros((rows, 1), np.uint64), w[:, :-1]])
        nxt = np.hstack([w[:, 1:], np.zeros((rows, 1), np.uint64)])
        lv = ((w << np.uint64(1)) | (prev >> np.uint64(31))) & M32   # funnel shift left by one
        rv = ((w >> np.uint64(1)) | (nxt << np.uint64(31))) & M32    # funnel shift right by one
        return lv, rv

    lv_a, rv_a = shifts(up)
    lv_b, rv_b = shifts(words)
    lv_c, rv_c = shifts(down)
    new = rule_bits(words, [lv_a, up, rv_a, lv_b, rv_b, lv_c, down, rv_c]) & M32
    tail = cols - 32 * (nw - 1)  # cells outside the grid stay dead
    if tail < 32:
        new[:, -1] &= np.uint64((1 << tail) - 1)
    return new


def test_boards_against_oracle():
    for rows, cols, seed in [(1, 1, 1), (5, 33, 2), (64, 96, 3), (100, 200, 4), (37, 1000, 5)]:
        board = (np.random.default_rng(seed).random((rows, cols)) < 0.3).astype(np.int32)
        words = pack(board)
        for _ in range(12):
            words = generation(words, cols)
        want = O.stencil2d_iterate(A.MSL_ST2_LIFE, board, 1, 0, 12)[0]
        assert np.array_equal(unpack(words, cols), want), (rows, cols)
