"""The C++ drop-in (include/branson_gb300_transport.hpp) compiles inside the
upstream code base and links against the CUDA library: the upstream headers
are used unmodified from the reference checkout, with the drop-in in place of
src/replicated_transport.h (tests/dropin/dropin_driver.cc)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(os.environ.get("BRANSON_REFERENCE", "/root/reference"), "src")


@pytest.mark.skipif(not os.path.isdir(REF), reason="upstream checkout not present")
def test_dropin_builds_against_upstream_headers(tmp_path):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    from branson_gb300 import build
    lib = build.build()
    out = tmp_path / "dropin_driver"
    cmd = ["g++", "-std=c++17", "-O1", "-w",
           "-I", os.path.join(ROOT, "oracle", "refstub"),
           "-I", os.path.join(ROOT, "oracle", "_ref", "cfg_g1"),
           "-I", REF, "-I", os.path.join(REF, "pugixml", "src"),
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "dropin_driver.cc"),
           os.path.join(ROOT, "oracle", "_ref", "pugixml.o"),
           lib, "-fopenmp", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert out.exists()
