"""Correctly rounded exp / log / pow reference values for the GPU accuracy test
of the table-driven transcendentals (mpmath, 120-bit working precision).

Inputs cover the argument ranges the NSW6 step produces (exponents of
saturation pressures, Roh-Satoh moments, temperature factors; logarithms of
mixing ratios and densities; the powers 2.47, 1.15, 0.75, 1.33, 1/3) plus a
wide log-uniform sweep.
"""
from __future__ import annotations

from pathlib import Path

import mpmath as mp
import numpy as np

HERE = Path(__file__).resolve().parent


def main() -> None:
    mp.mp.prec = 120
    rng = np.random.Generator(np.random.PCG64(4242))
    ex = np.concatenate([rng.uniform(-60, 40, 4000), rng.uniform(-1, 1, 2000), rng.uniform(-700, 700, 1000),
                         np.array([0.0, 1e-300, -1e-300, 1e-10, -1e-10, 0.6931471805599453, -0.6931471805599453])])
    lx = np.concatenate([10.0 ** rng.uniform(-30, 10, 4000), rng.uniform(0.5, 2.0, 2000),
                         1.0 + rng.uniform(-1e-3, 1e-3, 1000), np.array([1.0, 2.0, 0.75, 1.5, 1e-300, 1e300])])
    px = np.concatenate([10.0 ** rng.uniform(-20, -1, 2500), 10.0 ** rng.uniform(2, 7, 1000),
                         10.0 ** rng.uniform(-20, -3, 1000)])
    py = np.concatenate([rng.choice([2.47, 1.15, 0.75, 1.33, 0.33333333], 2500), np.full(1000, 1.33),
                         rng.uniform(-2.0, 3.0, 1000)])
    ey = np.array([float(mp.exp(mp.mpf(float(v)))) for v in ex])
    ly = np.array([float(mp.log(mp.mpf(float(v)))) for v in lx])
    pw = np.array([float(mp.power(mp.mpf(float(a)), mp.mpf(float(b)))) for a, b in zip(px, py)])
    np.savez_compressed(HERE / "fastmath_cr.npz", exp_x=ex, exp_y=ey, log_x=lx, log_y=ly, pow_x=px, pow_y=py,
                        pow_r=pw)


if __name__ == "__main__":
    main()
