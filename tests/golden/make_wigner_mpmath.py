"""Ground-truth Wigner-d values d^l_mn(beta_k) at l_max = 255 for the stable recursion.

Writes tests/golden/wigner_mpmath_lmax255.json: 240 samples (l, m, n, k) on the
l_max = 255 sampling grid beta_k = (2k+1) pi / 1024, weighted towards beta near pi
and l > 128 (where the reference recursion, fdcl_FFTSO3.cpp:127-194, loses its
seed d(l,l,l) = cos(beta/2)^(2l) to underflow), each evaluated with mpmath from
Wigner's explicit sum

  d^l_mn(b) = sqrt((l+m)!(l-m)!(l+n)!(l-n)!)
              * sum_s (-1)^(m-n+s) cos(b/2)^(2l+n-m-2s) sin(b/2)^(m-n+2s)
                      / ((l+n-s)! s! (m-n+s)! (l-m-s)!)

at 300 significant digits (the alternating sum cancels ~160 digits at l = 255)
and checked against a second evaluation at 360 digits.  The sign convention is
the reference's: it equals the reference recursion's values wherever those are
accurate (checked by tests/test_wigner_ground_truth.py against the oracle).

Run here (mpmath is not needed where the tests run):
    python tests/golden/make_wigner_mpmath.py
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "wigner_mpmath_lmax255.json")
L = 255
N = 2 * (L + 1)


def beta_k(k: int):
    import mpmath as mp
    return (2 * k + 1) * mp.pi / (4 * (L + 1))


def wigner_d_exact(l: int, m: int, n: int, k: int, dps: int):
    import mpmath as mp
    with mp.workdps(dps):
        b = beta_k(k)
        c, s = mp.cos(b / 2), mp.sin(b / 2)
        f = mp.factorial
        pre = mp.sqrt(f(l + m) * f(l - m) * f(l + n) * f(l - n))
        tot = mp.mpf(0)
        for t in range(0, 2 * l + 1):
            a, bb, cc = l + n - t, m - n + t, l - m - t
            if a < 0 or bb < 0 or cc < 0:
                continue
            term = c ** (2 * l + n - m - 2 * t) * s ** (m - n + 2 * t) / (f(a) * f(t) * f(bb) * f(cc))
            tot += -term if (m - n + t) & 1 else term
        return +(pre * tot)


def samples() -> list[tuple[int, int, int, int]]:
    rng = np.random.Generator(np.random.PCG64(255))
    near_pi = list(range(N - 8, N))          # beta within 8 grid steps of pi
    near_0 = list(range(0, 4))
    middle = sorted(int(x) for x in rng.choice(np.arange(4, N - 8), size=12, replace=False))
    out: list[tuple[int, int, int, int]] = []

    def mn(l: int, anti: bool, diag: bool):
        m = int(rng.integers(-l, l + 1))
        if anti:   # m + n small: the O(1) values near beta = pi
            n = int(np.clip(-m + rng.integers(-3, 4), -l, l))
        elif diag:  # m - n small: the O(1) values near beta = 0
            n = int(np.clip(m + rng.integers(-3, 4), -l, l))
        else:
            n = int(rng.integers(-l, l + 1))
        return m, n

    for i in range(130):                      # beta near pi, l > 128
        l = int(rng.integers(129, L + 1))
        out.append((l, *mn(l, anti=i % 2 == 0, diag=False), near_pi[i % len(near_pi)]))
    for i in range(40):                       # beta near 0, l > 128
        l = int(rng.integers(129, L + 1))
        out.append((l, *mn(l, anti=False, diag=i % 2 == 0), near_0[i % len(near_0)]))
    for i in range(58):                       # the rest of the grid, all degrees
        l = int(rng.integers(0, L + 1))
        out.append((l, *mn(l, anti=False, diag=False), middle[i % len(middle)]))
    for k in (N - 1, middle[3], 0):           # corners and the centre of the top degree
        for m, n in ((L, L), (L, -L), (-L, L), (0, 0)):
            out.append((L, m, n, k))
    return out


def main() -> None:
    import mpmath as mp
    rows = []
    for (l, m, n, k) in samples():
        v = wigner_d_exact(l, m, n, k, 300)
        v2 = wigner_d_exact(l, m, n, k, 360)
        if v != 0:
            assert abs(v - v2) <= abs(v) * mp.mpf(10) ** -40, (l, m, n, k)
        else:
            assert v2 == 0
        log10 = float(mp.log10(abs(v))) if v != 0 else -math.inf
        rows.append({"l": l, "m": m, "n": n, "k": k,
                     "value": float(v) if abs(v) > mp.mpf(10) ** -300 else 0.0,
                     "digits": mp.nstr(v, 30), "log10_abs": log10})
    doc = {"what": "d^l_mn(beta_k) at l_max = 255, beta_k = (2k+1) pi / 1024, the reference's sign convention, "
                   "from Wigner's explicit sum in mpmath at 300 digits (checked at 360); generated by "
                   "make_wigner_mpmath.py",
           "l_max": L, "samples": rows}
    with open(OUT, "w") as fh:
        json.dump(doc, fh, indent=0)
        fh.write("\n")
    print(f"wrote {len(rows)} samples to {OUT}")


if __name__ == "__main__":
    main()
