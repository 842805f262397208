"""Generate the minimax coefficients of atan used by the fan backprojector.

atan(t) ~= t * P(t^2) on |t| <= TMAX, P of degree DEG, fitted for minimum
maximum RELATIVE error with the Remez exchange algorithm (E. Remez, 1934;
see e.g. J.-M. Muller, "Elementary Functions", ch. 3) in float64 from the
mathematical function itself.  The kernel only uses it where every pixel of a
tile satisfies |r/d| <= TMAX (d > 0), i.e. fan angles up to ~31 degrees; other
tiles use atan2f.

    python gen_atan_poly.py  -> prints the C++ tables pasted into bp_tile.cuh

A tile takes the lowest degree whose range covers every pixel of the tile
(VARIANTS: (TMAX, DEG) pairs of about the same relative error, ~4e-8).
"""
import numpy as np

TMAX = 0.6
DEG = 5
VARIANTS = ((0.6, 5), (0.45, 4), (0.3, 3), (0.15, 2))


def remez(tmax=TMAX, deg=DEG, iters=80):
    n = deg + 2
    ts = tmax * (1 - np.cos(np.pi * np.arange(n) / (n - 1))) / 2
    ts[0] = tmax * 1e-3
    grid = np.linspace(tmax * 1e-4, tmax, 400001)
    c = None
    for _ in range(iters):
        A = np.zeros((n, n))
        b = np.ones(n)
        for i, t in enumerate(ts):
            at = np.arctan(t)
            A[i, :deg + 1] = [t ** (2 * k + 1) / at for k in range(deg + 1)]
            A[i, deg + 1] = (-1) ** i
        c = np.linalg.solve(A, b)[:deg + 1]
        e = (grid * np.polyval(c[::-1], grid ** 2) - np.arctan(grid)) / np.arctan(grid)
        s = np.sign(e)
        cuts = np.where(np.diff(s) != 0)[0]
        bounds = [0] + list(cuts + 1) + [len(grid)]
        idx = [a + int(np.argmax(np.abs(e[a:bb]))) for a, bb in zip(bounds[:-1], bounds[1:])]
        if len(idx) >= n:
            idx = sorted(sorted(idx, key=lambda j: -abs(e[j]))[:n])
            ts = grid[idx]
    err = float(np.max(np.abs((grid * np.polyval(c[::-1], grid ** 2) - np.arctan(grid)) / np.arctan(grid))))
    return c, err


if __name__ == "__main__":
    rows, errs = [], []
    for tmax, deg in VARIANTS:
        c, err = remez(tmax, deg)
        rows.append("{" + ", ".join(f"{v:.17e}" for v in list(c) + [0.0] * (5 - deg)) + "}")
        errs.append(f"|t| <= {tmax}: degree {deg}, max relative error {err:.2e}")
    print("// atan(t) ~= t*P(t^2) (Remez, degree in t^2): " + "; ".join(errs))
    print("ranges (atan_tmax):", ", ".join(f"{t}" for t, _ in VARIANTS))
    print("constexpr double kAtanPoly[%d][6] = {%s};" % (len(VARIANTS), ",\n    ".join(rows)))
