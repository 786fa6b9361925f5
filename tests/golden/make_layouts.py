"""Writes tests/golden/physx_layouts.json: sizeof/offsetof of the reference's
immediate-mode types, from tests/layout_probe.cpp built against the reference's
own headers.  Run where the reference sources exist."""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def physx_include():
    """The reference's include directory: $PHYSX_REFERENCE/include, else the
    source location the oracle/ref recipe names."""
    root = os.environ.get("PHYSX_REFERENCE")
    if not root:
        root = subprocess.check_output(["make", "-s", "-C", os.path.join(HERE, "..", "..", "oracle", "ref"), "print-physx"]).decode().strip()
    return os.path.join(root, "include")


if __name__ == "__main__":
    PHYSX_INCLUDE = physx_include()
    if not os.path.isdir(PHYSX_INCLUDE):
        sys.exit("reference headers not found")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "probe")
        subprocess.check_call(["g++", "-std=c++14", "-DPROBE_REFERENCE", "-DNDEBUG", "-Wno-invalid-offsetof", "-I", PHYSX_INCLUDE,
                               os.path.join(os.path.dirname(HERE), "layout_probe.cpp"), "-o", exe])
        out = subprocess.check_output([exe]).decode()
    open(os.path.join(HERE, "physx_layouts.json"), "w").write(out)
    print("wrote physx_layouts.json")
