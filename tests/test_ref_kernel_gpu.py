"""The oracle and the GPU drop-in pinned to the reference's own Monte-Carlo
kernel, run on the GPU from the reference's sources (oracle/mcref_harness.cu:
mc_kernel, src/mc.cu:83-197, with its own Sobol/xorshift set-up,
src/gen_rand.cuh:7-25 and src/mc.cu:366-454).

1. Value level (replay). The harness records every draw the reference's
   helpers make; the oracle's mc_kernel body (oracle/rc_unit_body.inc, the
   same text the oracle runs on Philox draws, which the GPU's rc_kernel
   matches bit for bit) replays them and must reproduce the reference's mcE
   bit for bit for every unit. That pins the kernel's control flow: the
   window ends (Q3), the photon scan with its sticky flags (Q4), the
   background clip, f_i, F and the final ratio; and the helpers' arguments
   (every Poisson mean and every binomial (n, p) must be the reference's).
   The helpers' own arithmetic is compared beside it: the oracle's log of
   the same uniform against drawTau (a few ulps: CUDA's logf against the
   project's own), the oracle's drawE formula on the same normal.
2. Distribution level. The reference's output and the drop-in's (gpda_mc,
   Philox counters) on the same bursts. For two states (the jump target is
   forced) a two-sample Kolmogorov-Smirnov test on the per-(burst, sample)
   values and a chi-square homogeneity test on their histograms, p > 1e-3.
   For three states and for static states (rates far below 1/T) the two
   differ by more than sampling noise, and not through the kernel, which the
   replay shows to be the oracle's: the reference's uniforms are not
   independent draws (each thread walks one scrambled Sobol dimension, and
   the dimensions repeat every 20,000 threads). There the test holds the
   distance to a stated margin (equivalence within the margin: KS D < 0.03,
   means within 0.02) and reports the lag-1 correlation of consecutive
   uniforms in the reference's recorded draws next to the oracle's Philox
   draws.

mc_kernel maps thread tidx to burst tidx >> (int)log2((double)R)
(src/mc.cu:101). Built here (CUDA 13, sm_103a) that shift can come out one
short of log2(R), and then the kernel gives each burst 2^shift samples and
its N * R threads reach bursts past N. The harness probes the shift on the
device and launches the kernel for the number of bursts that keeps every
thread on the bursts it was given; the comparisons use its 2^shift samples
per burst.

Skipped where the harness sources were not extracted (the reference tree is
not mounted where oracle/build_mcref.py ran).
"""
import numpy as np
import pytest

from gsmfretda_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mcref():
    import build_mcref
    if not build_mcref.available() and not build_mcref.extract():
        pytest.skip("reference kernel sources not extracted (oracle/_ref/mcref)")
    import mcref as _m
    _m.load()
    return _m


def _case(name):
    """(burst data, n, args) of one regime."""
    d = synth.photon_stream(B=2048, seed=21)
    rng = np.random.default_rng(5)
    if name == "2state":
        return d, 2, synth.pack_args([0.3, 0.72], [[0, 800.0], [1200.0, 0]])
    if name == "3state":                       # Q2: the dwell uses the chosen transition's rate
        return d, 3, synth.random_3state_args(rng)
    if name == "3state-broadening":            # drawE with V > 0
        a = synth.random_3state_args(rng).copy()
        a[9:12] = [3.0, 5.0, 4.0]
        return d, 3, a
    if name == "no-background":                # bg_dd_rate < 1e-4: f_i = floor(f_if + 0.5)
        return dict(d, bg_ad_rate=0.0, bg_dd_rate=0.0), 3, synth.random_3state_args(rng)
    if name == "slow":                         # Q1: rates below 1/s, unnormalised initial weights
        return d, 2, synth.pack_args([0.25, 0.8], [[0, 0.4], [0.7, 0]])
    if name == "fast":                         # Q3: tens of windows per burst
        return d, 3, synth.pack_args([0.2, 0.5, 0.85],
                                     [[0, 2e4, 3e4], [2.5e4, 0, 1.5e4], [1e4, 3e4, 0]])
    raise KeyError(name)


CASES = ["2state", "3state", "3state-broadening", "no-background", "slow", "fast"]


def test_thread_to_burst_shift(mcref):
    """The shift the reference kernel computes on this device, reported for
    R = 1 .. 1024; it is log2(R) or one short of it."""
    got = {1 << k: mcref.shift(1 << k) for k in range(11)}
    print("shift (int)log2((double)R) on this device:", got)
    for k in range(11):
        assert got[1 << k] in (k, k - 1), got


@pytest.mark.parametrize("name", CASES)
def test_oracle_replays_the_reference_kernel_bit_exact(orc, mcref, name):
    d, n, args = _case(name)
    m = orc.model()
    R = 8
    cap = 4096 if name == "fast" else 256
    ref, tape, tlen, reff = mcref.run(d, n, args, m, R, tape_cap=cap)
    assert tlen.max() <= cap, tlen.max()
    out, status, st = orc.rc_replay(d, n, args, m, reff, tape, tlen, ref)
    bad = np.nonzero(status)[0]
    assert st["exact"] == st["units"], (st, bad[:10], out[bad[:5]], ref[bad[:5]])
    assert st["lambda_mismatch"] == 0 and st["binom_arg_mismatch"] == 0, st
    assert st["tau_max_ulp"] <= 4, st                  # CUDA logf vs the project's log
    assert st["e_max_abs"] <= 2e-6, st                 # drawE formula, powf vs exp(log/6)
    kinds = np.unique(tape["tag"][tape["tag"] != 0] & 0xff)
    assert orc.TAPE_B in kinds and orc.TAPE_TAU in kinds
    if name != "no-background":
        assert orc.TAPE_P in kinds
    if name == "fast":
        assert np.mean(tlen) > 60                      # many windows per unit


def _dropin_values(d, n, args, R):
    from gsmfretda_gb300.mc import mc
    pdamc = mc(0, 2)
    pdamc.set_reSampleTimes(R)
    pdamc.set_seed(777)
    pdamc.init_data_gpu(d["istart"], d["start"], d["stop"], d["phCount"], d["times"].size,
                        d["burst_ad"], d["burst_dd"], d["T"], synth.sgdivsr(d), d["clk_p"],
                        d["bg_ad_rate"], d["bg_dd_rate"])
    sid = 0
    old = pdamc.set_nstates(n, sid)
    assert pdamc.set_params(n, sid, args)
    N = pdamc.setBurstBd(0, d["start"].size, sid)
    pdamc.init_randstate(N, sid)
    pdamc.set_params_buff(old, N, sid)
    pdamc.run_kernel(N, sid)
    while not pdamc.streamQuery(sid):
        pass
    ours = pdamc.hmcE(sid).reshape(-1).copy()
    pdamc.close()
    return ours


def _compare(ref, ours):
    from scipy import stats
    ks = stats.ks_2samp(ref, ours)
    edges = np.linspace(0.0, 1.0, 22)
    hr, _ = np.histogram(ref, edges)
    ho, _ = np.histogram(ours, edges)
    keep = (hr + ho) > 0
    chi = stats.chi2_contingency(np.stack([hr[keep], ho[keep]]))
    return ks, chi


def test_dropin_matches_the_reference_in_distribution(orc, mcref, gpda_lib):
    _, n, args = _case("2state")
    d = synth.photon_stream(B=16384, seed=23)
    m = orc.model()
    ref, _, _, reff = mcref.run(d, n, args, m, 16)
    ours = _dropin_values(d, n, args, reff)
    assert ours.size == ref.size
    ks, chi = _compare(ref, ours)
    print(f"2state: KS D={ks.statistic:.5f} p={ks.pvalue:.3g}; chi2 p={chi.pvalue:.3g}; "
          f"means {ref.mean():.5f} / {ours.mean():.5f}")
    assert ks.pvalue > 1e-3, ks
    assert chi.pvalue > 1e-3, chi


def _lag1(tape, tlen, cap):
    """Correlation of consecutive uniforms within each thread's draws."""
    a, b = [], []
    for t in range(tlen.size):
        rec = tape[t, :min(tlen[t], cap)]
        u = rec["d"][(rec["tag"] & 0xff) == 1]
        if u.size > 1:
            a.append(u[:-1])
            b.append(u[1:])
    a, b = np.concatenate(a), np.concatenate(b)
    return float(np.corrcoef(a, b)[0, 1]), a.size


@pytest.mark.parametrize("name", ["slow", "3state"])
def test_dropin_within_margin_of_the_reference(orc, mcref, gpda_lib, name):
    _, n, args = _case(name)
    d = synth.photon_stream(B=16384, seed=23)
    m = orc.model()
    ref, tape, tlen, reff = mcref.run(d, n, args, m, 16, tape_cap=256)
    ours = _dropin_values(d, n, args, reff)
    ks, chi = _compare(ref, ours)
    c_ref, npairs = _lag1(tape, tlen, 256)
    tape_o, tlen_o, _ = orc.rc_record(d, n, args, m, reff, 777, 256)
    c_ours, _ = _lag1(tape_o, tlen_o, 256)
    print(f"{name}: KS D={ks.statistic:.5f} p={ks.pvalue:.3g}; chi2 p={chi.pvalue:.3g}; "
          f"means {ref.mean():.5f} / {ours.mean():.5f}; lag-1 correlation of consecutive "
          f"uniforms: reference {c_ref:+.4f} ({npairs} pairs), Philox {c_ours:+.4f}")
    assert ks.statistic < 0.03
    assert abs(float(ref.mean()) - float(ours.mean())) < 0.02
    assert abs(c_ours) < 0.01
