"""The sweep schedule on the CPU.  Per-sweep launches (each stage-2 sweep and
each L-sweep as its own chain of launches on its own stream, the L-sweeps
waiting for their two producing stage-2 sweeps) hold the same cell solves as
one launch per step, address one output plane per sweep, and leave no race:
every two launches that touch the same trace line, output region or scratch
range, one of them writing, are ordered by the streams and events the library
uses.  The same holds for one launch per step with the per-shift streams of a
captured apply (fronts whose items each belong to one shifted decomposition
as one launch per shift on concurrent streams).  A small program
(tests/host/schedule_probe.cpp) is compiled with the library's schedule
builder (csrc/geometry.cpp) and run on the benchmark decompositions and on
small odd ones, with one to sixteen right-hand sides."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "l-sweeps-2d_gb300" / "csrc"


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    if not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("CUDA headers not found")
    out = tmp_path_factory.mktemp("sched") / "schedule_probe"
    cmd = [cxx, "-std=c++17", "-O2", str(ROOT / "tests" / "host" / "schedule_probe.cpp"), str(CSRC / "geometry.cpp"),
           "-I", str(ROOT / "include"), "-I", str(CSRC), "-I", str(cuda_inc), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("N,m,p,nrhs", [
    (2, 10, 4, 1), (3, 12, 5, 1), (5, 7, 2, 3), (6, 5, 1, 2), (3, 12, 5, 8), (5, 7, 2, 16),
    (4, 64, 10, 1),     # C1
    (8, 128, 16, 1),    # C2
    (8, 128, 16, 4),
    (16, 128, 20, 1),   # C3, one source
    (16, 128, 20, 16),  # C3, a batch of 16 sources
    (32, 128, 20, 1),   # C4
])
def test_concurrent_launches_have_no_race(probe, N, m, p, nrhs):
    r = subprocess.run([str(probe), str(N), str(m), str(p), str(nrhs)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    launches, steps, shift_launches = (int(t.split("=")[1]) for t in r.stdout.split()[1:4])
    assert steps <= shift_launches <= 4 * steps
    # stage 1, then four launches per stage-2 column and per stage-3 anti-diagonal
    assert steps == 1 + (N - 1) + (2 * N - 3)
    assert launches == 1 + 4 * (N - 1) + 4 * (2 * N - 3)


@pytest.mark.parametrize("slots", [4, 8, 16])
@pytest.mark.parametrize("N,m,p,nrhs", [(3, 12, 5, 1), (4, 16, 6, 2), (5, 7, 2, 8), (8, 128, 16, 16)])
def test_no_race_with_imposed_item_sizes(probe, N, m, p, nrhs, slots):
    """The same checks with every launch's items cut to 4, 8 or 16 slots (the
    tuner's candidates, LSW_FRONT_SHAPE): the items of a cell and their
    scratch change, the absence of races must not."""
    r = subprocess.run([str(probe), str(N), str(m), str(p), str(nrhs), str(slots)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
