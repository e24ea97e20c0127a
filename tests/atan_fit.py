"""Generator of the polynomial tables of the float atan2 filters in
axion-strings_gb300/csrc/axs_analysis.cu.

Both approximate atan(a) = a P(a^2) on a in [0, 1] (the octant-reduced
argument a = min(|x|,|y|) / max(|x|,|y|)); P minimises the largest absolute
error of a P(a^2) over a fine grid, found by Lawson's algorithm (C. L. Lawson,
"Contributions to the theory of linear least maximum approximation", 1961):
weighted least squares whose weights are multiplied by the current error
after every solve, which converges to the equal-ripple (minimax) solution.

  kAtanC  degree 7 in a^2, radians   (fast_atan2: background means)
  kTurnC  degree 5 in a^2, turns     (fast_turns: the string finder; the
          function divided by 2 pi, so the angle comes out in turns)

    python tests/atan_fit.py      prints both tables as C initialisers
"""
import numpy as np


def lawson(degree, scale=1.0, points=200001, iterations=60):
    """Coefficients c[0..degree] (float64) of P with a P(a^2) ~ atan(a) / scale."""
    a = np.linspace(0.0, 1.0, points)[1:]
    s = a * a
    target = np.arctan(a) / scale
    V = np.vander(s, degree + 1, increasing=True) * a[:, None]
    w = np.full(a.size, 1.0 / a.size)
    c = None
    for _ in range(iterations):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(V * sw[:, None], target * sw, rcond=None)
        err = np.abs(V @ c - target)
        w = w * err
        w /= w.sum()
    return c


def tables():
    return {"kAtanC": lawson(7), "kTurnC": lawson(5, scale=2.0 * np.pi)}


def as_c(name, c):
    vals = ", ".join("%.9ef" % np.float32(v) for v in c)
    return "__device__ constexpr float %s[%d] = {%s};" % (name, len(c), vals)


if __name__ == "__main__":
    for k, v in tables().items():
        print(as_c(k, v))
