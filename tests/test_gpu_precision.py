"""Mixed precision: FP16/BF16 storage of the analytic signals with FP32
accumulation, error against the FP64 CPU oracle in dB relative to the image
peak; the bar is -60 dB."""
import numpy as np
import pytest

from helpers import db_err, oracle_spec, run_host

pytestmark = pytest.mark.gpu

DB_BAR = -60.0


def _frames():
    from us_lab4a_gb300 import workloads
    return [("cf2d-pcf", workloads.cf2d(small=True)), ("plain2d", workloads.plain2d(small=True)),
            ("matrix3d", workloads.matrix3d(small=True))]


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("name,frame", _frames(), ids=[n for n, _ in _frames()])
def test_error_against_fp64_oracle(cuda, oracle_lib, name, frame, storage):
    from us_lab4a_gb300 import workloads
    fr = workloads.with_storage(frame, storage)
    rf = frame.make_rf_numpy()
    # FP64 oracle with element positions and grid in double.
    v64, _, _ = oracle_lib.process(oracle_spec(oracle_lib, fr.spec), rf, fr.grid_xyz, dtype=np.float64)
    v, _ = run_host(fr.spec, rf, fr.grid_xyz)
    err = db_err(v, v64)
    bar = {"f32": -100.0, "f16": DB_BAR, "bf16": DB_BAR}[storage]
    assert err <= bar, f"{name} {storage}: {err:.1f} dB"
