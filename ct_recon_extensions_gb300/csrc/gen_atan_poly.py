"""Generate the minimax polynomials of the fan backprojector's tile-relative
channel positions.

Within a tile, a pixel's fan angle is taken relative to the ray through the
tile's reference pixel: gamma = gamma0 + atan(t), where t is the tangent of
the angle between the two rays (small: |t| <= T for the whole tile).  atan is
a polynomial in z = t^2:

    atan(t) ~= t * A(z)          (minimum maximum RELATIVE error)

fitted on [0, T^2] with the Remez exchange algorithm (E. Remez, 1934; see
J.-M. Muller, "Elementary Functions", ch. 3) in float64 from the mathematical
function itself.  A tile takes the variant with the smallest T that covers all
its pixels (VARIANTS: T, degree of A); the degree is the lowest whose error,
times the largest angle of the range and the detector's dsd/ds (about 850
channels per radian), stays below about 2e-7 channels.

    python gen_atan_poly.py  -> prints the C++ tables pasted into bp_tile.cuh
"""
import numpy as np

VARIANTS = ((0.3, 4), (0.12, 3), (0.06, 2))


def remez_rel(f, zmax, deg, iters=60):
    """Coefficients c[0..deg] of P(z) = sum c[k] z^k minimising
    max |P(z) - f(z)| / |f(z)| on [0, zmax], and that maximum."""
    n = deg + 2
    zs = zmax * (1 - np.cos(np.pi * np.arange(n) / (n - 1))) / 2
    grid = np.linspace(0.0, zmax, 200001)
    c = None
    for _ in range(iters):
        A = np.zeros((n, n))
        b = f(zs)
        for i, z in enumerate(zs):
            A[i, :deg + 1] = [z ** k for k in range(deg + 1)]
            A[i, deg + 1] = (-1) ** i * f(z)
        c = np.linalg.solve(A, b)[:deg + 1]
        e = (np.polyval(c[::-1], grid) - f(grid)) / f(grid)
        s = np.sign(e)
        cuts = np.where(np.diff(s) != 0)[0]
        bounds = [0] + list(cuts + 1) + [len(grid)]
        idx = [a + int(np.argmax(np.abs(e[a:bb]))) for a, bb in zip(bounds[:-1], bounds[1:])]
        if len(idx) >= n:
            idx = sorted(sorted(idx, key=lambda j: -abs(e[j]))[:n])
            zs = grid[idx]
    err = float(np.max(np.abs((np.polyval(c[::-1], grid) - f(grid)) / f(grid))))
    return c, err


def atan_over_t(z):
    r = np.sqrt(np.maximum(z, 1e-300))
    return np.where(z > 0, np.arctan(r) / r, 1.0)


if __name__ == "__main__":
    arows, notes = [], []
    for tmax, da in VARIANTS:
        ca, ea = remez_rel(atan_over_t, tmax * tmax, da)
        arows.append("{" + ", ".join(f"{v:.17e}" for v in list(ca) + [0.0] * (4 - da)) + "}")
        notes.append(f"|t| <= {tmax}: atan degree {da} ({ea:.1e})")
    print("// " + "; ".join(notes))
    print("constexpr double kRelAtan[%d][5] = {%s};" % (len(VARIANTS), ",\n    ".join(arows)))
