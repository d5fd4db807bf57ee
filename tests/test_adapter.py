"""The C++ drop-in processors (include/usgb_sta_processor.hpp,
include/usgb_single_processor.hpp, include/usgb_two_medium_processor.hpp) compile inside
the reference's own headers, link libusgb.so, run through the reference's
ArrayProcessor interface and rethrow library errors as the reference's
exception types. Needs the reference sources (present where the fixtures are
made); the GPU part runs only where a GPU is present."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.ref import REF_SRC as REF


def _build(tmp_path):
    from us_lab4a_gb300 import build
    lib = build.build()
    shim = os.path.join(ROOT, "oracle", "refbuild", "shim")
    inc = [shim, f"{REF}/util", f"{REF}/fft", f"{REF}/user/processor", f"{REF}/user/acquisition",
           f"{REF}/user/configuration", REF, os.path.join(ROOT, "include")]
    srcs = [os.path.join(ROOT, "tests", "adapter", "adapter_main.cpp")] + [
        f"{REF}/util/{f}" for f in ("Log.cpp", "ParameterMap.cpp", "KeyValueFileReader.cpp")]
    exe = str(tmp_path / "adapter")
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-pthread"] + ["-I" + i for i in inc] + srcs + [
        lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_adapter_compiles_in_reference_tree_and_maps_errors(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120).stdout
    # Parameter checks run before any device work: the reference's exception type.
    assert "dead_zone InvalidValueException" in out and "Invalid dead zone" in out
    assert "tnrn_apod InvalidValueException Wrong rx apodization size: 7 (should be 8)." in out
    assert "tnrn_no_delays InvalidStateException Empty tx delay list." in out
    assert "tnrn_dead_zone InvalidValueException" in out and "deadZoneSamplesUp_" in out
    import torch
    for case in ("frame", "saft_frame", "tnrn_frame", "synthy_frame", "two_medium_frame", "two_medium_onetx_frame"):
        if torch.cuda.is_available():
            assert f"\n{case} ok" in "\n" + out, out
        else:
            # No device here: the CUDA failure surfaces as Lab::Exception.
            assert f"\n{case} Exception" in "\n" + out, out
