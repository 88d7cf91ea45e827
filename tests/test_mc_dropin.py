"""The C++ `mc` drop-in (include/gpda_mc.hpp): compiles and links against
libgpda.so with the reference's call sequence (CPU), and its results equal the
oracle's bit for bit (GPU)."""
import os
import subprocess

import numpy as np
import pytest

from gsmfretda_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dropin_exe(gpda_lib, tmp_path_factory):
    from gsmfretda_gb300._lib import LIB_PATH
    out = str(tmp_path_factory.mktemp("dropin") / "mc_dropin")
    libdir = os.path.dirname(LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "mc_dropin.cpp"), "-o", out,
           f"-L{libdir}", "-lgpda", f"-Wl,-rpath,{libdir}"]
    subprocess.check_call(cmd)
    return out


def test_dropin_compiles_against_reference_call_sequence(dropin_exe):
    assert os.access(dropin_exe, os.X_OK)


def write_input(path, d, n, args, R, nbins, seed, sid, cstart, cstop):
    B = d["start"].size
    with open(path, "wb") as f:
        np.array([B, d["burst_ad"].size], dtype=np.int64).tofile(f)
        np.array([n, R, nbins], dtype=np.int32).tofile(f)
        np.array([seed], dtype=np.uint64).tofile(f)
        np.array([d["clk_p"], d["bg_ad_rate"], d["bg_dd_rate"]], dtype=np.float32).tofile(f)
        np.array([sid, cstart, cstop], dtype=np.int32).tofile(f)
        for k in ("istart", "start", "stop"):
            d[k].astype(np.int64).tofile(f)
        d["phCount"].astype(np.int32).tofile(f)
        d["burst_ad"].astype(np.int64).tofile(f)
        d["burst_dd"].astype(np.int64).tofile(f)
        d["T"].astype(np.float32).tofile(f)
        synth.sgdivsr(d).astype(np.float32).tofile(f)
        np.asarray(args, dtype=np.float32).tofile(f)


@pytest.mark.gpu
def test_dropin_matches_oracle(dropin_exe, orc, tmp_path):
    d = synth.photon_stream(B=800, seed=61)
    n, R, nbins, seed, sid = 3, 4, 40, 777, 1
    args = synth.random_3state_args(np.random.default_rng(62))
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    # setBurstBd(100, 600): the reference simulates bursts [0, N) whatever the start (mc.cu:571)
    write_input(inp, d, n, args, R, nbins, seed, sid, 100, 600)
    subprocess.check_call([dropin_exe, inp, outp])
    raw = np.fromfile(outp, dtype=np.uint8)
    N = int(raw[:4].view(np.int32)[0])
    vals = raw[4:4 + 4 * N * R].view(np.float32).reshape(N, R)
    hist = raw[4 + 4 * N * R:].view(np.float32)
    assert N == 500
    m = orc.model(nbins=nbins)
    h_ref, e_ref = orc.run_refcompat(d, n, args, m, R, seed + sid, b0=0, b1=N)
    np.testing.assert_array_equal(vals.view(np.uint32), e_ref.view(np.uint32))
    np.testing.assert_array_equal(hist, h_ref.astype(np.float32))
