"""include/gbpx_immediate.h restates the byte layouts of the reference's
immediate-mode types; the layout probe built against it must print the same
sizeof/offsetof table as the probe built against the reference's headers
(tests/golden/physx_layouts.json)."""
import json
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_compat_header_layouts_match_reference():
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "physx_layouts.json")))
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "probe")
        subprocess.check_call(["g++", "-std=c++14", "-Wno-invalid-offsetof", "-I", os.path.join(ROOT, "include"),
                               os.path.join(ROOT, "tests", "layout_probe.cpp"), "-o", exe])
        ours = json.loads(subprocess.check_output([exe]).decode())
    assert ours == ref, {k: (ours.get(k), ref.get(k)) for k in set(ours) | set(ref) if ours.get(k) != ref.get(k)}
