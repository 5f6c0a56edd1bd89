"""Generates tests/golden/known_answers.json: closed-form known answers for the
step loop, computed with exact rational arithmetic (fractions) or closed-form
formulas, independently of the oracle and of the CUDA library.

Contents:
  * julia_div: Julia's float ``div(x, y)`` returns the exact truncated quotient
    of the two binary64 values (Julia Base, base/div.jl); it is used by
    update_particle_chunk! (src/chunks.jl:129-130). Computed here exactly.
  * chunk_index: (row, col) of points for a chunk grid, from the exact
    quotient and the clamp of index n+1 (src/chunks.jl:129-142).
  * capacity: chunk capacities (src/chunks.jl:32-34) of the benchmark grids.
  * lj_pair / harm_pair: two-particle forces from the closed forms
    (src/configs.jl:354-368, 389-397).
  * grid: rectangular_grid corner positions and box (src/init_states.jl:34-57).
  * invasions: rings with dyadic vertex coordinates (multiples of 1/64, so
    every binary64 operation of point_line_intersect lands on the exact
    comparison outcome) and the invasion list check_invasions!(system,
    ::Nothing) pushes (src/rings/integration.jl:378-470, 497-507), with the
    ray crossings decided in exact rational arithmetic.

Run: python tests/golden/make_golden.py
"""
import json
import math
import pathlib
from fractions import Fraction

OUT = pathlib.Path(__file__).resolve().parent / "known_answers.json"


def exact_div(x: float, y: float) -> float:
    q = Fraction(x) / Fraction(y)
    t = math.trunc(q)
    return float(t) if t != 0 else math.copysign(0.0, float(q))


def main():
    ans = {}
    cases = [(1.0, 0.1), (0.3, 0.1), (0.7, 0.1), (2.9999999999999996, 1.0), (3.0, 1.0), (-0.5, 1.0),
             (-1.5, 1.0), (43.3270350647418, 2.548649121455400), (10.0, 2.5), (1e-300, 1.0),
             (5.0, 0.1), (1084.6665937113297, 2.001229877696180), (7.0, 2.0), (0.1 * 3, 0.1),
             (123.456, 0.001), (1.0, 1.0 / 3.0), (2.0, 1.0 / 3.0)]
    ans["julia_div"] = [{"x": x, "y": y, "div": exact_div(x, y)} for x, y in cases]

    # chunk grid: box 10 x 6 at bottom-left (-1, 2), 5 cols x 3 rows
    L, H, blx, bly, cols, rows = 10.0, 6.0, -1.0, 2.0, 5, 3
    cl, ch = L / cols, H / rows
    pts = [(-1.0, 2.0), (9.0, 8.0), (-1.0, 8.0), (9.0, 2.0), (0.999, 7.999), (1.0, 6.0), (4.0, 5.0),
           (-1.2, 5.0), (4.0, 8.5), (-3.5, 5.0), (4.0, 1.0)]
    ci = []
    for x, y in pts:
        qr = exact_div((-y + bly) + H, ch)
        qc = exact_div(x - blx, cl)
        row = int(qr) + 1
        col = int(qc) + 1
        row -= 1 if row == rows + 1 else 0
        col -= 1 if col == cols + 1 else 0
        inside = 1 <= row <= rows and 1 <= col <= cols
        ci.append({"x": x, "y": y, "row": row, "col": col, "inside": inside})
    ans["chunk_grid"] = {"length": L, "height": H, "bl": [blx, bly], "cols": cols, "rows": rows}
    ans["chunk_index"] = ci

    def cap(cl, ch, r):
        nc = (math.ceil(0.5 * cl / r) + 1) * (math.ceil(0.5 * ch / r) + 1)
        return int(math.ceil(nc * 2))
    r_lj = 2 ** (1 / 6) / 2
    L1 = 32 * 2 * r_lj + r_lj * 0.4 * 33
    L3 = 2048 * 2 * r_lj + r_lj * 0.4 * 2049
    L2 = math.sqrt(262144 * math.pi / 0.70)
    ans["capacity"] = [
        {"name": "lj_1024", "chunk_l": L1 / 17, "r": r_lj, "cap": cap(L1 / 17, L1 / 17, r_lj)},
        {"name": "harm_262144", "chunk_l": L2 / 542, "r": 1.0, "cap": cap(L2 / 542, L2 / 542, 1.0)},
        {"name": "lj_4194304", "chunk_l": L3 / 1103, "r": r_lj, "cap": cap(L3 / 1103, L3 / 1103, r_lj)},
    ]

    lj = []
    for sigma, eps, d in [(1.0, 1.0, 2 ** (1 / 6)), (1.0, 1.0, 1.0), (1.0, 1.0, 1.5), (2.0, 4.0, 2.5)]:
        f = 4 * eps * (12 * sigma ** 12 / d ** 13 - 6 * sigma ** 6 / d ** 7)   # along +x on particle at +d
        lj.append({"sigma": sigma, "epsilon": eps, "d": d, "force_on_right": f})
    ans["lj_pair"] = lj
    hp = []
    for k_rep, k_atr, deq, dmax, d in [(10.0, 0.0, 2.0, 2.0, 1.5), (10.0, 2.0, 1.0, 1.2, 1.1), (10.0, 2.0, 1.0, 1.2, 1.3)]:
        if d > dmax:
            f = 0.0
        elif d < deq:
            f = -k_rep * (d / deq - 1)
        else:
            f = -k_atr * (d / deq - 1)
        hp.append({"k_rep": k_rep, "k_atr": k_atr, "dist_eq": deq, "dist_max": dmax, "d": d, "force_on_right": f})
    ans["harm_pair"] = hp

    r = r_lj
    ans["grid"] = {"nx": 32, "ny": 32, "offset": 0.4, "radius": r,
                   "first": [-r + r * (2 + 0.4), r * (0.4 + 1)],
                   "length": 32 * 2 * r + r * 0.4 * 33}
    ans["invasions"] = invasion_cases()
    OUT.write_text(json.dumps(ans, indent=1))
    print(f"wrote {OUT}")


def crosses(p, a, b):
    """point_line_intersect with exact rationals: the ray from p towards +x
    crosses edge a-b strictly inside both ranges."""
    dx, dy = b[0] - a[0], b[1] - a[1]
    ylo, yhi = (b[1], a[1]) if dy < 0 else (a[1], b[1])
    if dx == 0:
        return a[0] > p[0] and ylo < p[1] < yhi
    if dy == 0:
        return False
    x_inter = (dy * a[0] - dx * a[1] + dx * p[1]) / dy
    xlo, xhi = (b[0], a[0]) if dx < 0 else (a[0], b[0])
    return x_inter > p[0] and xlo < x_inter < xhi and ylo < p[1] < yhi


def invasion_cases():
    import random
    rnd = random.Random(2024)
    cases = []
    for _ in range(3):
        nr, n = 6, 7
        rings = []
        for _ in range(nr):
            cx, cy = Fraction(rnd.randint(-192, 192), 64), Fraction(rnd.randint(-192, 192), 64)
            pts = []
            for k in range(n):
                ang = 2 * math.pi * k / n + rnd.random() * 0.3
                rad = 1.0 + rnd.random() * 0.5
                pts.append((cx + Fraction(round(rad * math.cos(ang) * 64), 64),
                            cy + Fraction(round(rad * math.sin(ang) * 64), 64)))
            rings.append(pts)
        out = []
        for r1 in range(nr):
            for r2 in range(r1 + 1, nr):
                for a, b in ((r1, r2), (r2, r1)):
                    for i, p in enumerate(rings[a]):
                        c = sum(crosses(p, rings[b][e], rings[b][(e + 1) % n]) for e in range(n))
                        if c % 2:
                            out.append([a + 1, b + 1, a * n + i + 1])
        cases.append({"rings_pos": [[[float(x), float(y)] for x, y in r] for r in rings], "invasions": out})
    return cases


if __name__ == "__main__":
    main()
