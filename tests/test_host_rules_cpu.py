"""Host-side march rules, no GPU: tests/host/face_rules_check.cpp is compiled
with the library's host set-up (anacor_public_gb300/csrc/reflection_setup.cpp)
and run.  It checks, for random reflections, that every face rule that can be
a leg's exit face marches in the octant of the leg's direction (the octant
field a leg reads), that the count axis steps by exactly +-1, and that the
field march's skip multiplier keeps every skip inside the box the distance
field proves uniform."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "anacor_public_gb300", "csrc")


def test_face_rules_octants_and_skips():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "face_rules_check")
        cmd = [gxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I", CSRC,
               "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "host", "face_rules_check.cpp"),
               os.path.join(CSRC, "reflection_setup.cpp"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
