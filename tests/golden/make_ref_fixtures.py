"""Writes reference_compiled.npz: outputs of the reference's own transform code, compiled here.

The reference's sources are compiled unmodified by oracle/ref.mk (against the
Eigen-API subset in oracle/ref_shim/) and called through oracle/ref.py.  The
inputs are synthesised by the oracle's inverse from seeded coefficients
(tests/conftest.py generators), so any host can rebuild them without the
reference; the fixture holds what the reference returned for them:

  l16_*   l_max = 16 (the CPU-runnable 34^3 case): the full forward outputs of
          FFTSO3_complex / FFTSO3_real / FFTS2_complex / FFTS2_real, the point
          inverses at seeded angles, and wigner_d at one beta;
  l127_*  l_max = 127 (the 256^3 FP64 case): the forward outputs of
          FFTSO3_complex / FFTSO3_real at NSAMPLE seeded coefficient indices,
          and their per-degree norms ||F^l||.

Run (needs the reference's source tree, a few minutes):
    python tests/golden/make_ref_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from conftest import s2_coeffs, so3_coeffs  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import ref  # noqa: E402

NSAMPLE = 2048
SEEDS = {"so3c": 1601, "so3r": 1602, "s2c": 1603, "s2r": 1604, "l127c": 12701, "l127r": 12702}


def points(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.stack([rng.uniform(-np.pi, np.pi, n), rng.uniform(0.05, np.pi - 0.05, n),
                     rng.uniform(-np.pi, np.pi, n)], axis=1)


def per_l_norms(F, L):
    return np.array([np.linalg.norm(F[l * (4 * l * l - 1) // 3:(l + 1) * (4 * (l + 1) ** 2 - 1) // 3])
                     for l in range(L + 1)])


def main():
    if not ref.available():
        raise SystemExit("the compiled reference is unavailable (no reference source tree)")
    out = {}
    L, N = 16, 34
    F = so3_coeffs(L, SEEDS["so3c"])
    out["l16_so3_complex"] = ref.so3_forward_complex(L, orc.so3_inverse_complex_grid(L, F).reshape(N, N, N))
    Fr = so3_coeffs(L, SEEDS["so3r"], complex_=False)
    out["l16_so3_real"] = ref.so3_forward_real(L, orc.so3_inverse_real_grid(L, Fr).reshape(N, N, N))
    S = s2_coeffs(L, SEEDS["s2c"])
    out["l16_s2_complex"] = ref.s2_forward_complex(L, orc.s2_inverse_complex_grid(L, S).reshape(N, N))
    Sr = s2_coeffs(L, SEEDS["s2r"], complex_=False)
    out["l16_s2_real"] = ref.s2_forward_real(L, orc.s2_inverse_real_grid(L, Sr).reshape(N, N))
    P = points(8, 1605)
    out["l16_points"] = P
    out["l16_so3_complex_points"] = np.array([ref.so3_inverse_complex_point(L, F, *p) for p in P])
    out["l16_so3_real_points"] = np.array([ref.so3_inverse_real_point(L, Fr, *p) for p in P])
    out["l16_s2_complex_points"] = np.array([ref.s2_inverse_complex_point(L, S, p[1], p[0]) for p in P])
    out["l16_s2_real_points"] = np.array([ref.s2_inverse_real_point(L, Sr, p[1], p[0]) for p in P])
    out["l16_wigner_d_beta"] = np.array(0.7)
    out["l16_wigner_d"] = ref.wigner_d(0.7, L)

    L, N = 127, 256
    n = orc.so3_ncoeff(L)
    idx = np.sort(np.random.Generator(np.random.PCG64(12703)).choice(n, NSAMPLE, replace=False))
    out["l127_index"] = idx
    F = so3_coeffs(L, SEEDS["l127c"])
    G = ref.so3_forward_complex(L, orc.so3_inverse_complex_grid(L, F).reshape(N, N, N))
    out["l127_so3_complex"] = G[idx]
    out["l127_so3_complex_norms"] = per_l_norms(G, L)
    Fr = so3_coeffs(L, SEEDS["l127r"], complex_=False)
    G = ref.so3_forward_real(L, orc.so3_inverse_real_grid(L, Fr).reshape(N, N, N))
    out["l127_so3_real"] = G[idx]
    out["l127_so3_real_norms"] = per_l_norms(G, L)
    out["seeds"] = np.array([SEEDS[k] for k in sorted(SEEDS)])
    path = os.path.join(HERE, "reference_compiled.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
