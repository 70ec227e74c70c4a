"""The drop-in boundary from a compiled C++ caller.

tests/cpp/green_main.cpp is the reference's test executable
(cusrc/main.cu:1-10) with the library's header: g++ must compile and link it
against libgrtm_gb300.so as it stands (CPU).  On the GPU, the executable's own
call -- green("../cusrc/example/crust1.0.txt", "out4.txt", "signal.txt") from
a build directory beside cusrc/, as the reference lays it out -- must write the
oracle's files, and a call on the reference's demo input must write files that
match the reference's golden outputs."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "green_main.cpp")


def _build(tmp_path):
    import grtm_cuda_gb300 as g
    lib = g.lib()._name
    exe = str(tmp_path / "green_main")
    cmd = ["g++", "-O1", "-Wall", "-Wno-write-strings", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           lib, "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_caller_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
    nm = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
    assert "green" in [ln.split()[-1] for ln in nm.splitlines() if ln.strip()]   # resolved from the library


def _run(exe, cwd, *args):
    env = dict(os.environ, GRT_PRECISION="fp64")
    r = subprocess.run([exe, *args], cwd=cwd, capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_reference_caller_writes_the_oracle_files(tmp_path, oracle):
    """main.cu's own call, from build/ beside cusrc/example/crust1.0.txt."""
    import grtm_cuda_gb300 as g
    exe = _build(tmp_path)
    ex = tmp_path / "cusrc" / "example"
    ex.mkdir(parents=True)
    shutil.copyfile(os.path.join(GOLDEN, "example_crust1.0_input.txt"), ex / "crust1.0.txt")
    build = tmp_path / "build"
    build.mkdir()
    _run(exe, build)
    # the oracle on the same file: the reference's grid and k rule, the FP64
    # library's basis (equal to the reference's where that is well conditioned)
    job = oracle.parse(str(ex / "crust1.0.txt"))
    oracle.setup(job, job.dt, job.log2n, job.t0, job.taper, fix=oracle.STABLE)
    spec, sig = oracle.run(job, [job.dist0])
    w_ref, t_ref = spec[0], sig[0]
    w, t = g.read_table(build / "out4.txt", complex_pairs=True), g.read_table(build / "signal.txt")
    assert w.shape == w_ref.shape == (2048, 30) and t.shape == t_ref.shape == (2048, 30)
    for c in range(15):
        assert np.linalg.norm(t[:, c] - t_ref[:, c]) <= 1e-9 * np.linalg.norm(t_ref[:, c]), c
        assert np.linalg.norm(w[:, c] - w_ref[:, c]) <= 1e-9 * np.linalg.norm(w_ref[:, c]), c
    assert np.abs(w[:, 15:]).max() == 0 and np.abs(t[:, 15:]).max() == 0


@pytest.mark.gpu
def test_reference_caller_on_the_demo_matches_golden(tmp_path, golden, oracle):
    """The demo input (demo/input.txt) through the compiled caller; the files
    against the reference's own outputs demo/oname_{w,t}.txt (the defined
    bins, as the Python file-interface test compares them)."""
    import grtm_cuda_gb300 as g
    import test_gpu_parity as P
    exe = _build(tmp_path)
    ow, ot = str(tmp_path / "w.txt"), str(tmp_path / "t.txt")
    _run(exe, tmp_path, os.path.join(GOLDEN, "demo_input.txt"), ow, ot)
    job = oracle.parse(os.path.join(GOLDEN, "demo_input.txt"))
    oracle.setup(job, job.dt, job.log2n, job.t0, job.taper)
    w = g.read_table(ow, complex_pairs=True)
    assert w.shape == (2048, 30)
    assert np.array_equal(w[job.nw + 1:], np.conj(w[job.nw - 1:0:-1]))
    for c in range(15):
        assert P._masked_time_err(w[:, c], golden["spec"], golden["sig"], job, c) < 5e-6, c
