"""The GPU codecs' device functions (psychopath_gb300/csrc/dev_compact.cuh),
compiled for the host with the same floating-point rules as the device
build (no contraction, IEEE division and square root) and a __fdividef that
errs by up to its documented 2 ulps at random, against the oracle on seeded
triples over the whole f32 range, special values, near-tie directions for
encode_precise and random codes for the decoders
(tests/compact_device_logic.cpp).  This pins the fast paths' decision rules
-- fluv32's integer filter, encode_precise's f32 ranking with f64 cosines
on near ties, the 40/48-bit codes in 32-bit halves -- without a GPU; the GPU
tests then check the device build itself."""
import os
import shutil
import subprocess

import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_device_codec_logic_on_host(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    oracle.build()
    exe = str(tmp_path / "compact_device_logic")
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math",
                    os.path.join(HERE, "compact_device_logic.cpp"), oracle.LIB_PATH,
                    "-Wl,-rpath," + os.path.dirname(oracle.LIB_PATH), "-o", exe], check=True)
    r = subprocess.run([exe, "400000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if "checked" in l]
    assert len(lines) == 13 and all(l.endswith(" 0 mismatches") for l in lines), r.stdout
