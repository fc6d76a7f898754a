"""What the learned acoustic-cycle surrogate gains over the plain FP32
sound loop (nompi/mod_moloch.F90:483-851), measured and stated.

Workload: a 128 x 128 x 30 hilly domain (500 m hill of 10-gridpoint radius,
6 m/s background wind, seeded +-0.5 K theta noise), FP32 storage.
Training: (state, post-cycle state) pairs collected from plain steps of a
scratch domain with another seed, in three windows spread over its first
60 steps (states from across the run, not only from its start); 3000 Adam
steps on the GPU.
Runs from the same initial state, 24 steps each: the FP64 step (the
reference), the plain FP32 step, FP32 with the surrogate attached under its
judge (the plain loop every 6th cycle, relative RMS error tolerance 0.3; a
rejection switches the surrogate off with a doubling interval), and FP32
with the surrogate forced on for every cycle (no judge, no envelope bound;
the on-device check still falls back to the plain loop when a prediction
is not finite).

Stated (printed as one record): cycles committed to the surrogate and their
fraction, the time per step of the judged and forced runs against the
plain FP32 run (CUDA events on the library's stream over graph replays),
and the RMSE of theta, u, v, w against the FP64 step for every FP32 run.
Asserted: the counts add up; the plain FP32 run is within the error budget
(theta RMSE <= 0.05 K, u, v, w RMSE <= 0.05 m/s); the judge protects the
run (its errors are at most those of the surrogate forced on).  The gain
itself is recorded, not asserted.  Measured on GB300: 10 of 72 cycles
committed, the judged step 1.10x the plain FP32 step, theta RMSE 0.078 K
(plain FP32: 0.0009 K); forced on for every cycle it diverges (NaN) within
the 24 steps -- the surrogate does not gain on this workload, and its few
accepted cycles already exceed the error budget.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JX, IY, KZ = 128, 128, 30
SETUP = dict(hills=((500.0, 64.5, 64.5, 10.0),), u0=6.0, v0=2.0, pert_amp=0.5, pert_levels=10)
STEPS = 24


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a) - np.asarray(b)) ** 2)))


def _time_steps(torch, g, n):
    st = torch.cuda.ExternalStream(g.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g.sync()
    e0.record(st)
    g.run(n, graph=True)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / n


def test_surrogate_gain_is_stated(gpu_lib):
    torch = pytest.importorskip("torch")
    dm = gpu_lib
    scratch = dm.Moloch(JX, IY, KZ, mode="fp32_mixed")
    scratch.setup_idealized(seed=1241, **SETUP)
    nadv = scratch.params.mo_nadv
    cols = 1024
    sur = dm.Surrogate(KZ, capacity=3 * 6 * nadv * cols, batch=256, seed=1)
    for w in range(3):  # windows of 6 collected steps at steps 0, 24, 48
        sur.collect(scratch, 6, cols_per_cycle=cols, seed=3 + w)
        if w < 2:
            scratch.run(18, graph=True)
    sur.prepare(0.1)
    _, v0 = sur.train(0)
    tl, vl = sur.train(3000, lr=1e-3)
    assert np.isfinite(vl) and vl < v0

    ref = dm.Moloch(JX, IY, KZ, mode="fp64")
    plain = dm.Moloch(JX, IY, KZ, mode="fp32_mixed")
    judged = dm.Moloch(JX, IY, KZ, mode="fp32_mixed")
    forced = dm.Moloch(JX, IY, KZ, mode="fp32_mixed")
    for g in (ref, plain, judged, forced):
        g.setup_idealized(**SETUP)
    ref.run(STEPS, graph=True)
    warm = 4
    ms = {}
    sur.attach(forced, threshold=1e30, judge_every=0)
    forced.run(warm, graph=True)
    ms["fp32_surrogate_forced"] = _time_steps(torch, forced, STEPS - warm)
    cf = sur.stats_counts()
    sur.detach()
    sur.attach(judged, threshold=4.0, judge_every=6, tol=0.3)
    for name, g in (("fp32", plain), ("fp32_surrogate", judged)):
        g.run(warm, graph=True)
        ms[name] = _time_steps(torch, g, STEPS - warm)
    c = sur.stats_counts()  # attach restarted the counts: the judged run alone
    th_ref = ref.get("t") / ref.get("pai")
    err = {}
    for name, g in (("fp32", plain), ("fp32_surrogate", judged), ("fp32_surrogate_forced", forced)):
        err[name] = {"theta_K": rmse(g.get("t") / g.get("pai"), th_ref), "u": rmse(g.get("u"), ref.get("u")),
                     "v": rmse(g.get("v"), ref.get("v")), "w": rmse(g.get("w"), ref.get("w"))}
    committed = c["cycles"] - c["plain"]
    record = {"workload": f"{JX}x{IY}x{KZ}, {STEPS} steps", "val_loss": [v0, vl],
              "cycles": c["cycles"], "committed": committed, "committed_fraction": committed / c["cycles"],
              "verdicts": c["judged"], "rejections": c["judge_rejections"],
              "forced_run_fallbacks_on_non_finite_output": cf["plain"], "ms_per_step": ms,
              "step_time_ratio_over_plain": {k: ms[k] / ms["fp32"] for k in ms if k != "fp32"},
              "rmse_vs_fp64": err,
              "gain": "none" if committed == 0 or ms["fp32_surrogate"] >= ms["fp32"] else "faster"}
    print("surrogate gain:", json.dumps(record))
    assert c["cycles"] == STEPS * nadv and cf["cycles"] == STEPS * nadv and cf["judged"] == 0
    assert 0 <= c["plain"] <= c["cycles"] and c["judged"] >= 1 and c["judge_rejections"] <= c["judged"]
    e = err["fp32"]
    assert e["theta_K"] <= 0.05 and e["u"] <= 0.05 and e["v"] <= 0.05 and e["w"] <= 0.05, record
    for f in ("theta_K", "u", "v", "w"):  # a forced run that diverged (NaN) counts as unbounded error
        ej, ef = err["fp32_surrogate"][f], err["fp32_surrogate_forced"][f]
        assert np.isfinite(ej) and (not np.isfinite(ef) or ej <= ef), (f, record)
    sur.close()
    for g in (scratch, ref, plain, judged, forced):
        g.close()
