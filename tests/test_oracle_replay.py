"""The replay machinery that pins the oracle's mc_kernel body to the
reference's own kernel output (tests/test_ref_kernel_gpu.py), checked on the
CPU: the oracle's own Philox draws written in the tape format must replay to
the oracle's ref-compat values bit for bit, and a planted change in a tape
(a binomial variate, a draw out of order, a cut tape, a wrong Poisson mean)
must show up in exactly the unit it was planted in."""
import numpy as np
import pytest

from gsmfretda_gb300 import synth


def _data(bg=True):
    d = synth.photon_stream(B=400, seed=21)
    if not bg:
        d = dict(d, bg_ad_rate=0.0, bg_dd_rate=0.0)
    return d


@pytest.mark.parametrize("n,bg,V", [(2, True, 0.0), (3, True, 0.0), (3, True, 4.0), (3, False, 0.0)])
def test_recorded_philox_draws_replay_bit_exact(orc, n, bg, V):
    d = _data(bg)
    rng = np.random.default_rng(5)
    if n == 3:
        args = synth.random_3state_args(rng).copy()
    else:
        args = synth.pack_args([0.3, 0.72], [[0, 800.0], [1200.0, 0]])
    args[n * n:] = V
    m = orc.model()
    R = 8
    tape, tl, mcE = orc.rc_record(d, n, args, m, R, 1234, 256)
    assert tl.max() <= 256
    _, e = orc.run_refcompat(d, n, args, m, R, 1234)
    np.testing.assert_array_equal(mcE.view(np.uint32), e.reshape(-1).view(np.uint32))
    out, status, st = orc.rc_replay(d, n, args, m, R, tape, tl, mcE)
    assert st["exact"] == st["units"] == 400 * R, st
    assert st["lambda_mismatch"] == 0 and st["binom_arg_mismatch"] == 0
    assert st["tau_max_ulp"] == 0 and st["e_max_abs"] == 0.0
    np.testing.assert_array_equal(out.view(np.uint32), mcE.view(np.uint32))
    kinds = set(np.unique(tape["tag"][tape["tag"] != 0] & 0xff).tolist())
    assert {orc.TAPE_U, orc.TAPE_TAU, orc.TAPE_N, orc.TAPE_E, orc.TAPE_B} <= kinds
    assert (orc.TAPE_P in kinds) == bg


def test_planted_changes_are_caught_in_their_unit(orc):
    d = _data()
    args = synth.random_3state_args(np.random.default_rng(6))
    m = orc.model()
    R = 4
    tape, tl, mcE = orc.rc_record(d, 3, args, m, R, 99, 256)
    kind = tape["tag"] & 0xff
    # a binomial variate that is not the one drawn (a unit whose F > 0)
    t1 = tape.copy()
    cand = [u for u in range(tl.size) if mcE[u] > 0 and np.any(kind[u, :tl[u]] == orc.TAPE_B)]
    u1 = cand[3]
    j = int(np.nonzero(kind[u1, :tl[u1]] == orc.TAPE_B)[0][0])
    t1[u1, j]["i"] += 1
    _, s1, st1 = orc.rc_replay(d, 3, args, m, R, t1, tl, mcE)
    assert np.nonzero(s1)[0].tolist() == [u1] and s1[u1] == 1
    # a draw of the wrong kind where the body wants a uniform
    t2 = tape.copy()
    t2[u1, 0]["tag"] = orc.TAPE_N
    _, s2, _ = orc.rc_replay(d, 3, args, m, R, t2, tl, mcE)
    assert np.nonzero(s2)[0].tolist() == [u1] and s2[u1] == 3
    # a cut tape
    tl3 = tl.copy()
    tl3[u1] = 300
    _, s3, _ = orc.rc_replay(d, 3, args, m, R, tape, tl3, mcE)
    assert np.nonzero(s3)[0].tolist() == [u1] and s3[u1] == 2
    # a Poisson mean that is not the body's tdiff * rate
    t4 = tape.copy()
    up = [u for u in range(tl.size) if np.any(kind[u, :tl[u]] == orc.TAPE_P)][0]
    jp = int(np.nonzero(kind[up, :tl[up]] == orc.TAPE_P)[0][0])
    t4[up, jp]["d"] *= 1.5
    _, s4, st4 = orc.rc_replay(d, 3, args, m, R, t4, tl, mcE)
    assert st4["lambda_mismatch"] == 1 and st4["exact"] == st4["units"]
