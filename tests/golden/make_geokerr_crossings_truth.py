"""Writes tests/golden/geokerr_crossings_truth.npz: the first six equatorial
crossings (u and the azimuth change from the start) of near-critical and
ordinary rays leaving a camera at r = 50 M, theta = 80 deg, computed at 40
digits by quadrature (oracle/geokerr_cf_mp.py, crossings): the truth for the
library's crossings by Jacobi amplitude (np_geokerr_disk_crossings_*) and
for the renderer's near-critical rays.

Near-critical rays: Carter constants on the critical curve of spherical
photon orbits (radius r_ph between the prograde and retrograde orbits),
l(r) = -(r^3 - 3 r^2 + a^2 r + a^2) / (a (r - 1)),
q2(r) = r^3 (4 a^2 - r (r - 3)^2) / (a^2 (r - 1)^2), with l moved by a
relative 1e-10 .. 1e-3 to either side (escaping and captured rays), at
a = 0.9, 0.998, 0.5 and -0.7; ordinary rays from a seeded box of (l, q2);
outgoing starts (su = -1) for a few.  The Taylor restatement's crossings
(oracle.geokerr_crossings) seed the truth's Newton steps.

    python tests/golden/make_geokerr_crossings_truth.py
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from oracle import geokerr_cf_mp as cfmp  # noqa: E402

K = 6
U0, MU0, UFAR = 0.02, math.cos(math.radians(80.0)), 1e-3


def critical(a, r):
    l = -(r ** 3 - 3 * r * r + a * a * r + a * a) / (a * (r - 1))
    q2 = r ** 3 * (4 * a * a - r * (r - 3) ** 2) / (a * a * (r - 1) ** 2)
    return l, q2


def allowed(a, l, q2):
    return q2 + (a * a - l * l - q2) * MU0 * MU0 - a * a * MU0 ** 4 >= 0


def main():
    rng = np.random.default_rng(7)
    rows = []
    for a in (0.9, 0.998, 0.5, -0.7):
        r_pro = 2 * (1 + math.cos(2 / 3 * math.acos(-abs(a))))
        r_ret = 2 * (1 + math.cos(2 / 3 * math.acos(abs(a))))
        cases = []
        while len(cases) < 7:
            l, q2 = critical(a, rng.uniform(min(r_pro, r_ret), max(r_pro, r_ret)))
            d = 10.0 ** rng.uniform(-10, -3) * (1 if len(cases) % 2 else -1)
            l = l * (1 + d)
            if q2 > 0 and allowed(a, l, q2):
                cases.append((l, q2, 1.0))
        while len(cases) < 9:
            l, q2 = rng.uniform(-8, 8), rng.uniform(0.5, 60)
            if allowed(a, l, q2):
                cases.append((l, q2, 1.0 if len(cases) == 7 else -1.0))
        for l, q2, su in cases:
            sm = float(rng.choice([-1.0, 1.0]))
            n_o, xu_o, _ = oracle.geokerr_crossings(U0, MU0, a, l, q2, su, sm, UFAR, K)
            out = cfmp.crossings(U0, MU0, a, l, q2, su, sm, UFAR, K=K, guess=list(xu_o[:max(n_o, 0)]))
            if out is None:
                continue
            st, xs, ph = out
            xu = np.zeros(K)
            xphi = np.zeros(K)
            xu[:len(xs)] = [float(x) for x in xs]
            xphi[:len(ph)] = [float(x) for x in ph]
            rows.append((a, l, q2, su, sm, st, len(xs), xu, xphi))
            print(a, l, q2, su, st, len(xs), flush=True)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "geokerr_crossings_truth.npz"),
                        a=np.array([r[0] for r in rows]), l=np.array([r[1] for r in rows]),
                        q2=np.array([r[2] for r in rows]), su=np.array([r[3] for r in rows]),
                        sm=np.array([r[4] for r in rows]),
                        status=np.array([r[5] for r in rows], dtype=np.int32),
                        n=np.array([r[6] for r in rows], dtype=np.int32),
                        xu=np.array([r[7] for r in rows]), xphi=np.array([r[8] for r in rows]),
                        u0=U0, mu0=MU0, u_far=UFAR)


if __name__ == "__main__":
    main()
