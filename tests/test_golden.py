"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py from
the oracle): the oracle must reproduce them bit for bit (regression pin),
and the CUDA path must match them (FP64_EXACT: rel. L2 <= 1e-13)."""
import os

import numpy as np
import pytest

from tests.conftest import rel_l2

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
from tests.golden.make_golden import CASES, CHECKSUM_CASE, FULL, PROBES, checksums  # noqa: E402


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(oracle_mod, name):
    jx, iy, kz, steps, opts = CASES[name]
    ref = np.load(os.path.join(HERE, name + ".npz"))
    o = oracle_mod.Oracle(oracle_mod.make_cfg(jx, iy, kz, **opts))
    for s in range(1, steps + 1):
        o.step(s)
    for f in FULL:
        assert np.array_equal(o.get(f), ref[f]), f


def test_oracle_reproduces_golden_checksums(oracle_mod):
    name, jx, iy, kz, steps = CHECKSUM_CASE
    ref = np.load(os.path.join(HERE, name + ".npz"))
    o = oracle_mod.Oracle(oracle_mod.make_cfg(jx, iy, kz))
    for s in range(1, steps + 1):
        o.step(s)
    for f in FULL:
        a = o.get(f)
        assert np.array_equal(checksums(a), ref[f + "_sums"]), f
        pr = np.array([a[p] if a.ndim == 3 else a[p[1], p[2]] for p in PROBES])
        assert np.array_equal(pr, ref[f + "_probes"]), f


def _gpu_opts(opts):
    prm, ideal = {}, {}
    for k, v in opts.items():
        if k in ("hills", "u0", "v0", "pert_amp", "pert_levels", "seed"):
            ideal[k] = v
        elif k == "divfilter":
            prm["mo_divfilter"] = int(v)
        elif k == "filterpai":
            prm["do_filterpai"] = int(v)
        elif k == "filtertheta":
            prm["do_filtertheta"] = int(v)
        elif k == "rotllr":
            prm["rotllr"] = int(v)
    return prm, ideal


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("mode", ["fp64_exact", "fp64"])
def test_gpu_matches_golden(gpu_lib, name, mode):
    jx, iy, kz, steps, opts = CASES[name]
    ref = np.load(os.path.join(HERE, name + ".npz"))
    prm, ideal = _gpu_opts(opts)
    g = gpu_lib.Moloch(jx, iy, kz, mode=mode, **prm)
    g.setup_idealized(**ideal)
    for s in range(1, steps + 1):
        g.moloch(s)
    tol = 1e-13 if mode == "fp64_exact" else 1e-11
    for f in FULL:
        assert rel_l2(g.get(f), ref[f]) <= tol, f


@pytest.mark.gpu
def test_gpu_matches_golden_checksums(gpu_lib):
    name, jx, iy, kz, steps = CHECKSUM_CASE
    ref = np.load(os.path.join(HERE, name + ".npz"))
    g = gpu_lib.Moloch(jx, iy, kz, mode="fp64_exact")
    g.setup_idealized()
    for s in range(1, steps + 1):
        g.moloch(s)
    for f in FULL:
        a = g.get(f)
        np.testing.assert_allclose(checksums(a), ref[f + "_sums"], rtol=1e-13, atol=0)
        pr = np.array([a[p] if a.ndim == 3 else a[p[1], p[2]] for p in PROBES])
        np.testing.assert_allclose(pr, ref[f + "_probes"], rtol=1e-13, atol=0)
