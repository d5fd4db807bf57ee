"""Image post-processing (usgb_post_*): the envelope along image columns and
the conversion to decibels, against the oracle's restatement of
HilbertEnvelope::calculate and Util::linearToDecibels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ENV_TOL = 1e-5     # of the envelope maximum (FP32 FFTs against FP64)
DB_TOL = 1e-4      # dB, where neither side is at the floor


@pytest.mark.parametrize("ncols,nrows", [(37, 300), (8, 1024), (3, 2049)])
def test_envelope_matches_oracle(cuda, oracle_lib, ncols, nrows):
    import torch
    from us_lab4a_gb300.post import PostProcessor
    rng = np.random.default_rng(ncols * 1000 + nrows)
    t = np.arange(nrows)
    img = (np.cos(2 * np.pi * 0.07 * t)[None, :] * rng.uniform(0.5, 2.0, (ncols, 1))
           + 0.1 * rng.standard_normal((ncols, nrows))).astype(np.float32)
    ref = oracle_lib.envelope(img.astype(np.float64))
    with PostProcessor(nrows) as post:
        x = torch.as_tensor(img, device=cuda)
        env = post.envelope(x).cpu().numpy()
        post.envelope(x, out=x)  # in place
        same = x.cpu().numpy()
    assert np.abs(env - ref).max() <= ENV_TOL * np.abs(ref).max()
    assert np.array_equal(env, same)


def test_envelope_of_a_real_path_image(cuda, oracle_lib):
    """The reference shows the real-RF (SCF) image as an envelope in dB."""
    import torch
    from helpers import run_host
    from us_lab4a_gb300 import workloads
    from us_lab4a_gb300.post import PostProcessor
    fr = workloads.plain2d(small=True, seed=5)
    fr.spec.real_path, fr.spec.coherence = True, "scf"
    v, _ = run_host(fr.spec, fr.make_rf_numpy(), fr.grid_xyz)
    ref = oracle_lib.envelope(v.astype(np.float64))
    with PostProcessor(v.shape[1]) as post:
        env = post.envelope(torch.as_tensor(v, device=cuda)).cpu().numpy()
    assert np.abs(env - ref).max() <= ENV_TOL * np.abs(ref).max()


@pytest.mark.parametrize("min_db", [-60.0, -20.0])
def test_decibels_match_oracle(cuda, oracle_lib, min_db):
    import torch
    from us_lab4a_gb300.post import PostProcessor
    rng = np.random.default_rng(3)
    img = np.abs(rng.standard_normal((50, 70))).astype(np.float32) ** 4
    img[3, 5] = 0.0
    ref = oracle_lib.linear_to_decibels(img, min_db)
    with PostProcessor(70) as post:
        x = torch.as_tensor(img, device=cuda)
        got = post.decibels(x, min_db).cpu().numpy()
        z = torch.zeros((4, 70), device=cuda)
        zeros = post.decibels(z, min_db).cpu().numpy()
    floor = (ref == min_db)
    assert np.array_equal(floor, got == min_db)
    assert np.abs(got[~floor] - ref[~floor]).max() <= DB_TOL
    assert abs(got.max()) <= 1e-5  # v * (1 / max) rounds to 1 within an ulp, as in the reference
    assert np.all(zeros == min_db)
