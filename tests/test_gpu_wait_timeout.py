"""The delay-and-sum's bounded waits, made to run out on purpose.

Every mbarrier wait of the staged delay-and-sum kernels gives up after a limit
(2 s by default) instead of waiting forever; the warp records the timeout in
the context's error word and the kernel winds down once its bulk copies in
flight have landed. The test hook usgb_set_wait_test shortens the limit and
makes the window producer of every pixel tile leave one stage unarmed, so the
consumers' wait for that stage runs out: no fault, no hang, the host reads
USGB_ERR_DEVICE_TIMEOUT, and the next frame on the same context is correct."""
import numpy as np
import pytest

from helpers import oracle_spec, rel_err

pytestmark = pytest.mark.gpu

WAIT_US = 2000   # 2 ms per bounded wait while the hook is on


@pytest.mark.parametrize("variant,skip", [(1, 3), (2, 1), (2, 5), (3, 2)])
def test_wait_runs_out_then_clean_frame(cuda, oracle_lib, variant, skip):
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    from us_lab4a_gb300.errors import DeviceTimeoutException
    fr = workloads.cf2d(small=True)
    rf_np = fr.make_rf_numpy()
    rf = torch.as_tensor(rf_np, device=cuda)
    grid = torch.as_tensor(fr.grid_xyz, device=cuda)
    v = torch.empty(fr.grid_xyz.shape[:2], device=cuda)
    f = torch.empty_like(v)
    with StaEngine(fr.spec) as eng:
        eng.set_stream(torch.cuda.current_stream())
        eng.set_das_variant(variant)
        eng.set_grid_device(grid)
        eng.set_wait_test(WAIT_US, skip)
        eng.process_device(rf, v, f)
        with pytest.raises(DeviceTimeoutException):
            eng.synchronize()
        # The host path reports it too.
        with pytest.raises(DeviceTimeoutException):
            eng.set_grid(fr.grid_xyz)
            eng.process_host(rf_np)
        # Hook off: the same context forms the frame correctly.
        eng.set_wait_test(0, 0)
        eng.set_grid_device(grid)
        eng.process_device(rf, v, f)
        eng.synchronize()
    vo, fo, _ = oracle_lib.process(oracle_spec(oracle_lib, fr.spec), rf_np, fr.grid_xyz, dtype=np.float32)
    assert rel_err(v.cpu().numpy(), vo) <= 1e-5
    assert np.abs(f.cpu().numpy() - fo).max() <= 1e-3


def test_limit_alone_does_not_fire(cuda):
    """A short limit without a skipped stage is not a failure: the stages
    arrive well within 2 ms on a small frame."""
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    fr = workloads.cf2d(small=True)
    with StaEngine(fr.spec) as eng:
        eng.set_das_variant(3)
        eng.set_grid(fr.grid_xyz)
        eng.set_wait_test(WAIT_US, 0)
        v, f = eng.process_host(fr.make_rf_numpy())
    assert np.isfinite(v).all()
