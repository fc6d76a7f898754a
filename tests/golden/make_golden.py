"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

The reference cannot be run (Fortran, no compiler on these machines), so
these fixtures pin the oracle against regressions and give the GPU tests a
fixed target; they are not outputs of the reference itself.

    python tests/golden/make_golden.py      # rewrites tests/golden/*.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle  # noqa: E402

FULL = ("u", "v", "w", "pai", "t", "qv", "ps")
CASES = {
    # name: (jx, iy, kz, steps, cfg options)
    "defaults_16x12x8": (16, 12, 8, 3, {}),
    "options_13x11x7": (13, 11, 7, 2, dict(divfilter=True, filterpai=True, filtertheta=True, rotllr=False,
                                            hills=((300.0, 6.0, 5.0, 2.5),), u0=4.0, v0=-2.0)),
}
# larger run kept as checksums only: the reference defaults, 20 steps
CHECKSUM_CASE = ("defaults_100x100x30", 100, 100, 30, 20)
PROBES = ((0, 0, 0), (29, 49, 49), (15, 99, 0), (5, 7, 93), (29, 0, 99))


def checksums(a):
    a = np.asarray(a, dtype=np.float64)
    w = np.arange(a.size, dtype=np.float64).reshape(a.shape) % 7 + 1
    return np.array([a.sum(), np.abs(a).sum(), (a * a).sum(), (w * a).sum()])


def run_case(jx, iy, kz, steps, opts):
    o = oracle.Oracle(oracle.make_cfg(jx, iy, kz, **opts))
    for s in range(1, steps + 1):
        o.step(s)
    return o


def main():
    oracle.build()
    for name, (jx, iy, kz, steps, opts) in CASES.items():
        o = run_case(jx, iy, kz, steps, opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **{f: o.get(f) for f in FULL},
                            meta=np.array([jx, iy, kz, steps]))
        o.close()
    name, jx, iy, kz, steps = CHECKSUM_CASE
    o = run_case(jx, iy, kz, steps, {})
    out = {}
    for f in FULL:
        a = o.get(f)
        out[f + "_sums"] = checksums(a)
        out[f + "_probes"] = np.array([a[p] if a.ndim == 3 else a[p[1], p[2]] for p in PROBES])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array([jx, iy, kz, steps]), **out)
    o.close()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
