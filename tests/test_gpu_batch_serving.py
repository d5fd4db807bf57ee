"""Batched launches and the serving loop: every frame's image is the same
alone and in a mixed-size batch (identical kernels and arithmetic, so the
images are compared bit for bit; the stated tolerance, 1e-5 of the image
maximum, is the fallback bar)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(frame, cuda, das_config):
    """The frame alone on the staged kernel (every delay-and-sum kernel gives
    the same bits; the staged kernel's tiles have 4, 8 or 16 rows)."""
    import torch
    from us_lab4a_gb300 import StaEngine
    rows, stage_bytes, stages = das_config
    with StaEngine(frame.spec) as eng:
        eng.set_stream(torch.cuda.current_stream())
        eng.set_das_variant(1, rows if rows in (4, 8, 16) else 4, stage_bytes, stages)
        eng.set_grid_device(torch.as_tensor(frame.grid_xyz, device=cuda))
        v = torch.empty(frame.grid_xyz.shape[:2], device=cuda)
        f = torch.empty_like(v)
        eng.process_device(torch.as_tensor(frame.make_rf_numpy(), device=cuda), v, f)
        eng.synchronize()
        return v.cpu().numpy(), f.cpu().numpy()


@pytest.mark.parametrize("variant,rows", [(1, 4), (2, 4), (3, 4), (3, 8), (4, 4), (4, 7), (4, 8)])
@pytest.mark.parametrize("use_graph", [False, True])
@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_batch_equals_frames_alone(cuda, use_graph, storage, variant, rows):
    """Every batched kernel form, including two points per thread (variant 4:
    64 x 8 tiles on 8 consumer warps, 64 x 14 on 14, 64 x 16 on 16)."""
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    from us_lab4a_gb300.batch import Batch, BatchItem
    frames = workloads.mixed(num_frames=7, small=True, storage=storage)
    cfg = (rows, 16384, 2)
    stream = torch.cuda.current_stream()
    batch = Batch(max_frames=16, max_elements=16)
    batch.set_das_config(*cfg, variant=variant)
    engines, items = [], []
    for fr in frames:
        eng = StaEngine(fr.spec)
        eng.set_stream(stream)
        eng.set_grid_device(torch.as_tensor(fr.grid_xyz, device=cuda))
        engines.append(eng)
        v = torch.full(fr.grid_xyz.shape[:2], -1.0, device=cuda)
        items.append(BatchItem(eng, torch.as_tensor(fr.make_rf_numpy(), device=cuda), v, torch.empty_like(v)))
    # Twice: the second run replays the captured graph with fresh descriptors
    # (a different subset and order of frames).
    for sel in (list(range(7)), [5, 0, 3]):
        for i in sel:
            items[i].value.fill_(-1.0)
        batch.run([items[i] for i in sel], stream, use_graph=use_graph)
        batch.synchronize()
        for i in sel:
            va, fa = _alone(frames[i], cuda, cfg)
            vb, fb = items[i].value.cpu().numpy(), items[i].factor.cpu().numpy()
            assert np.array_equal(va, vb), (i, np.abs(va - vb).max())
            assert np.array_equal(fa, fb)
    batch.close()
    for e in engines:
        e.close()


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_batch_equals_long_frames_alone(cuda, storage):
    """Two frames of A-scans of 4096 samples at 8x (32768 upsampled) and one
    of at most 512 samples at 4x: alone, a long frame's preparation runs one
    512-thread block an SM and parks the real parts in tensor memory (one
    store pass of whole samples), the short frame's runs 128-thread blocks
    with two store passes; in the batch the longest A-scan makes the blocks
    512 threads, one an SM, and every frame's real parts are parked. The
    images agree bit for bit."""
    import torch
    from dataclasses import replace
    from us_lab4a_gb300 import StaEngine, workloads
    from us_lab4a_gb300.batch import Batch, BatchItem
    frames = workloads.mixed(num_frames=3, small=True, storage=storage)
    for fr in frames[:2]:
        fr.spec = replace(fr.spec, num_samples=4096, upsampling=8)
    assert frames[2].spec.num_samples <= 512
    cfg = (4, 16384, 2)
    stream = torch.cuda.current_stream()
    engines, items = [], []
    with Batch(max_frames=4, max_elements=16) as batch:
        batch.set_das_config(*cfg, variant=1)
        for fr in frames:
            eng = StaEngine(fr.spec)
            eng.set_stream(stream)
            eng.set_grid_device(torch.as_tensor(fr.grid_xyz, device=cuda))
            engines.append(eng)
            v = torch.full(fr.grid_xyz.shape[:2], -1.0, device=cuda)
            items.append(BatchItem(eng, torch.as_tensor(fr.make_rf_numpy(), device=cuda), v, torch.empty_like(v)))
        batch.run(items, stream, use_graph=False)
        batch.synchronize()
        for fr, it in zip(frames, items):
            va, fa = _alone(fr, cuda, cfg)
            vb, fb = it.value.cpu().numpy(), it.factor.cpu().numpy()
            assert np.abs(va).max() > 0
            assert np.array_equal(va, vb), np.abs(va - vb).max()
            assert np.array_equal(fa, fb)
    for e in engines:
        e.close()


def test_serving_results_same_alone_and_in_mix(cuda):
    import torch
    from us_lab4a_gb300 import workloads
    from us_lab4a_gb300.serving import Request, ServingLoop, poisson_arrivals
    frames = workloads.mixed(num_frames=12, small=True, storage="f16")
    arrivals = poisson_arrivals(len(frames), rate=2000.0, seed=3)
    reqs = [Request(i, fr.spec, fr.grid_xyz, torch.as_tensor(fr.make_rf_numpy()).pin_memory(), float(t))
            for i, (fr, t) in enumerate(zip(frames, arrivals))]
    loop = ServingLoop(hbm_budget_bytes=2 << 30, max_batch=4, max_elements=16, das_config=(4, 16384, 2))
    stats = loop.run(reqs)
    loop.close()
    assert stats["frames"] == len(frames) and stats["batches"] >= 3
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    for r, fr in zip(reqs, frames):
        va, fa = _alone(fr, cuda, (4, 16384, 2))
        assert np.abs(r.value - va).max() <= 1e-5 * np.abs(va).max()
        assert np.array_equal(r.value, va) and np.array_equal(r.factor, fa)


def test_serving_admission_respects_budget(cuda):
    import torch
    from us_lab4a_gb300 import workloads
    from us_lab4a_gb300.serving import Request, ServingLoop
    frames = workloads.mixed(num_frames=6, small=True, storage="f16")
    reqs = [Request(i, fr.spec, fr.grid_xyz, torch.as_tensor(fr.make_rf_numpy()).pin_memory(), 0.0)
            for i, fr in enumerate(frames)]
    loop = ServingLoop(hbm_budget_bytes=1, max_batch=4, max_elements=16)
    sizes = [loop._slot_bytes(r.spec, r.grid_xyz) for r in reqs]
    loop.budget = max(sizes)  # the largest frame fits, but never with all the others
    stats = loop.run(reqs)
    loop.close()
    assert stats["peak_resident_bytes"] <= loop.budget
    assert stats["batches"] > 1 and stats["mean_batch"] < len(reqs)
    assert all(r.value is not None for r in reqs)
