"""Generates tests/golden/known_answers.json: known-answer vectors for the
oracle, computed here by independent pure-Python restatements of the
reference shader formulas (integer arithmetic with explicit 32-bit wrap,
float32 arithmetic through numpy) and by hand-derived cases.

The reference repository ships no tests or golden data, and its shaders
cannot run without a Vulkan ray-query device, so these vectors are derived
from the shader source text:
  tea             initSeeds.comp:7-19
  halton          raygenPrimary.comp:11-22
  sobol2d         raygenShadow.comp:22-40
  morton aila32   computeMortonCodesAila32.comp:39-88 (hand-built rays)
  pixel table     Ray/PixelTable.cpp:33-93
  reinhard        interpolateColors.comp:10-57 (float64 reference values)

Run: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

M32 = 0xFFFFFFFF
f32 = np.float32


def tea(v0: int, v1: int, rounds: int = 16) -> int:
    s0 = 0
    for _ in range(rounds):
        s0 = (s0 + 0x9E3779B9) & M32
        v0 = (v0 + ((((v1 << 4) & M32) + 0xA341316C) & M32 ^ ((v1 + s0) & M32) ^ (((v1 >> 5) + 0xC8013EA4) & M32))) & M32
        v1 = (v1 + ((((v0 << 4) & M32) + 0xAD90777D) & M32 ^ ((v0 + s0) & M32) ^ (((v0 >> 5) + 0x7E95761E) & M32))) & M32
    return v0


def halton(i: int, base: int) -> float:
    r = f32(0.0)
    f = f32(1.0) / f32(base)
    j = i
    while j > 0:
        r = f32(r + f32(f * f32(j % base)))
        j //= base
        f = f32(f / f32(base))
    return float(r)


def sobol2d(i: int):
    r1 = r2 = 0
    v1, v2 = 1 << 31, 3 << 30
    while i > 0:
        if i & 1:
            r1 ^= v1
            r2 ^= (v2 << 1) & M32
        v1 = v1 | (v1 >> 1)
        v2 = v2 ^ (v2 >> 1)
        i >>= 1
    return float(f32(r1) / f32(4294967296.0)), float(f32(r2) / f32(4294967296.0))


def aila32(ia, ib) -> int:
    """Bit layout written out from the shader, MSB first."""
    order = []
    for lvl in (6, 5, 4, 3):
        order += [("a", 0, lvl), ("a", 1, lvl), ("a", 2, lvl)]
    order += [("b", 0, 3), ("b", 1, 3), ("b", 2, 3)]
    order += [("a", 0, 2), ("a", 1, 2), ("a", 2, 2)]
    order += [("b", 0, 2), ("b", 1, 2), ("b", 2, 2)]
    order += [("a", 0, 1), ("a", 1, 1), ("a", 2, 1)]
    order += [("b", 0, 1), ("b", 1, 1), ("b", 2, 1)]
    order += [("a", 0, 0), ("a", 1, 0), ("a", 2, 0)]
    order += [("b", 0, 0), ("b", 1, 0)]
    assert len(order) == 32
    k = 0
    for pos, (w, ax, lvl) in zip(range(31, -1, -1), order):
        v = ia[ax] if w == "a" else ib[ax]
        k |= ((v >> lvl) & 1) << pos
    return k


def morton_case(origin, direction, smin, ssize):
    o = np.array(origin, f32)
    d = np.array(direction, f32)
    a = np.clip((o - np.array(smin, f32)) / np.array(ssize, f32), f32(0), f32(1)).astype(f32)
    ln = f32(np.sqrt(f32(f32(f32(d[0] * d[0]) + f32(d[1] * d[1])) + f32(d[2] * d[2]))))
    nd = (d / ln).astype(f32)
    b = ((nd + f32(1)) * f32(0.5)).astype(f32)
    ia = [int(f32(x * f32(127))) for x in a]
    ib = [int(f32(x * f32(15))) for x in b]
    return aila32(ia, ib)


def pixel_table(w: int, h: int):
    idx = 0
    bh, bw = h & ~7, w & ~7
    md = max(bw, bh)
    for s in (1, 2, 4, 8, 16):
        md |= md >> s
    md = (md + 1) >> 1
    w8, h8 = bw >> 3, bh >> 3
    i2p = [0] * (w * h)
    for i in range(md * md):
        tx = ty = 0
        val, bit = i, 1
        while val:
            if val & 1:
                tx |= bit
            if val & 2:
                ty |= bit
            bit += bit
            val >>= 2
        if tx < w8 and ty < h8:
            for inner in range(64):
                ix = (inner & 1) | ((inner & 4) >> 1) | ((inner & 16) >> 2)
                iy = ((inner & 2) >> 1) | ((inner & 8) >> 2) | ((inner & 32) >> 3)
                i2p[idx] = (ty * 8 + iy) * w + tx * 8 + ix
                idx += 1
    for px in range(bw):
        for py in range(bh, h):
            i2p[idx] = px + py * w
            idx += 1
    for py in range(h):
        for px in range(bw, w):
            i2p[idx] = px + py * w
            idx += 1
    assert idx == w * h
    return i2p


def reinhard64(c, key, white):
    R = [[0.5141364, 0.265068, 0.0241188], [0.3238786, 0.67023428, 0.1228178], [0.16036376, 0.06409157, 0.84442666]]
    X, Y, Z = (sum(R[r][k] * c[k] for k in range(3)) for r in range(3))
    x, y = X / (X + Y + Z), Y / (X + Y + Z)
    lp = Y * key / 0.5
    L = lp * (1 + lp / (white * white)) / (1 + lp)
    X2, Y2, Z2 = L * x / y, L, L * (1 - x - y) / y
    M = [[2.5651, -1.0217, 0.0753], [-1.1665, 1.9777, -0.2543], [-0.3986, 0.0439, 1.1892]]
    return [M[r][0] * X2 + M[r][1] * Y2 + M[r][2] * Z2 for r in range(3)]


def main():
    out = {}
    out["tea"] = [[i, f, tea(i, f)] for i in (0, 1, 2, 255, 65535, 123456, 4294967295) for f in (1, 2, 77)]
    out["halton"] = [[i, b, halton(i, b)] for i in (0, 1, 2, 3, 4, 7, 100, 1023) for b in (2, 3)]
    out["sobol2d"] = [[i, *sobol2d(i)] for i in range(0, 17)]
    cases = []
    smin, ssize = [0.0, 0.0, 0.0], [1.0, 1.0, 1.0]
    for o, d in [((0, 0, 0), (1, 0, 0)), ((1, 1, 1), (1, 0, 0)), ((0.5, 0.25, 0.75), (0, 1, 0)),
                 ((2, -1, 0.3), (-1, -1, -1)), ((0.1, 0.9, 0.5), (0.3, -0.4, 0.866))]:
        cases.append([list(o), list(d), smin, ssize, morton_case(o, d, smin, ssize)])
    # hand-derived: origin at min, direction +x -> ib = (15, 7, 7)
    assert cases[0][4] == (1 << 19) | (7 << 11) | (7 << 5) | 3
    out["morton_aila32"] = cases
    out["pixel_table"] = {f"{w}x{h}": pixel_table(w, h) for (w, h) in [(16, 16), (13, 10), (8, 3), (24, 17)]}
    out["reinhard"] = [[c, k, wp, reinhard64(c, k, wp)] for c in ([0.5, 0.5, 0.5], [1.0, 0.2, 0.1], [0.01, 0.3, 2.0])
                       for k, wp in ((0.6, 2.0), (0.4, 1.0))]
    out["sincos_2pi"] = [[r, math.sin(2 * math.pi * r), math.cos(2 * math.pi * r)]
                         for r in (0.0, 0.1, 0.125, 0.25, 0.3, 0.5, 0.6, 0.75, 0.875, 0.999999)]
    path = Path(__file__).with_name("known_answers.json")
    path.write_text(json.dumps(out, indent=1))
    print(path)


if __name__ == "__main__":
    main()
