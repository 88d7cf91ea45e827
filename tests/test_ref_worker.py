"""The reference's own GPU thread, gpuWorker::run (src/gpuWorker.cpp:38-88),
compiled unchanged from the reference's sources against the drop-in header
include/gpda_mc.hpp (with stand-ins for the headers it includes but does not
use for this path: args.pb.h, tools.hpp), linked with libgpda.so (CPU), and
run through the stream hand-off of streamWorker::run with its results equal
to the oracle's bit for bit (GPU).

The sources come from the reference tree where it is mounted, else from the
copy oracle/build_mcref.py extracted into oracle/_ref/worker/; the test is
skipped where neither exists. Nothing of the reference is committed.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from gsmfretda_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUBS = os.path.join(ROOT, "tests", "cpp", "ref_worker_stubs")


def _worker_sources():
    import build_mcref
    for d in (os.path.join(build_mcref.REF_ROOT, "src"), build_mcref.WORKER_DIR):
        if all(os.path.exists(os.path.join(d, f)) for f in build_mcref.WORKER_FILES):
            return d, build_mcref.WORKER_FILES
    return None, None


@pytest.fixture(scope="module")
def worker_exe(gpda_lib, tmp_path_factory):
    src, files = _worker_sources()
    if src is None:
        pytest.skip("the reference's gpuWorker sources are not available here")
    from gsmfretda_gb300._lib import LIB_PATH
    tmp = tmp_path_factory.mktemp("refworker")
    # the reference's files and the stand-ins side by side: gpuWorker.hpp's
    # #include "mc.hpp" resolves in its own directory first
    for f in files:
        shutil.copyfile(os.path.join(src, f), tmp / f)
    for f in os.listdir(STUBS):
        shutil.copyfile(os.path.join(STUBS, f), tmp / f)
    out = str(tmp / "ref_gpuworker")
    libdir = os.path.dirname(LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++17", "-pthread", "-I", str(tmp), "-I", os.path.join(ROOT, "include"),
           str(tmp / "gpuWorker.cpp"), os.path.join(ROOT, "tests", "cpp", "ref_gpuworker_main.cpp"),
           "-o", out, f"-L{libdir}", "-lgpda", f"-Wl,-rpath,{libdir}"]
    subprocess.check_call(cmd)
    return out


def test_reference_gpuworker_compiles_against_the_dropin(worker_exe):
    assert os.access(worker_exe, os.X_OK)


@pytest.mark.gpu
def test_reference_gpuworker_results_equal_the_oracle(worker_exe, orc, tmp_path):
    from test_mc_dropin import write_input
    d = synth.photon_stream(B=700, seed=63)
    n, R, nbins, seed, sid = 3, 8, 30, 4242, 1
    args = synth.random_3state_args(np.random.default_rng(64))
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, d, n, args, R, nbins, seed, sid, 0, 600)
    subprocess.check_call([worker_exe, inp, outp], timeout=180)
    raw = np.fromfile(outp, dtype=np.uint8)
    N = int(raw[:4].view(np.int32)[0])
    vals = raw[4:4 + 4 * N * R].view(np.float32).reshape(N, R)
    hist = raw[4 + 4 * N * R:].view(np.float32)
    assert N == 600
    m = orc.model(nbins=nbins)
    h_ref, e_ref = orc.run_refcompat(d, n, args, m, R, seed + sid, b0=0, b1=N)
    np.testing.assert_array_equal(vals.view(np.uint32), e_ref.view(np.uint32))
    np.testing.assert_array_equal(hist, h_ref.astype(np.float32))
