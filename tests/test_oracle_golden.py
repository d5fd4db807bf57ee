"""Pins the CPU oracle to the reference: its own golden vectors (test/*.h5 of
the reference, extracted into tests/golden/reference_vectors.npz) with the
tolerances of src/user/method/TestMethod.cpp:59-71, and the outputs of the
reference processors themselves (tests/golden/reference_frames.npz)."""
import numpy as np
import pytest

# TestMethod.cpp tolerances.
HILBERT_MAX_RELATIVE_ABS_ERROR = 1.0e-15
INTERPOLATOR_MAX_RELATIVE_ABS_ERROR = 1.0e-14
INTERPOLATOR_LP_FILTER_TRANSITION_WIDTH = 0.45
KAISER_MAX_RELATIVE_ABS_ERROR = 1.0e-15
FFT_MAX_RELATIVE_ABS_ERROR = 1.0e-12


def test_hilbert_transform_golden(oracle_lib, golden_vectors):
    """TestMethod::testHilbertTransform (TestMethod.cpp:681-744), analytic part."""
    x = golden_vectors["hilbert_x"]
    yc = oracle_lib.hilbert(x)
    max_abs = np.abs(yc).max()
    err = np.maximum(np.abs(yc.real - golden_vectors["hilbert_yr"]), np.abs(yc.imag - golden_vectors["hilbert_yi"]))
    assert err.max() / max_abs <= HILBERT_MAX_RELATIVE_ABS_ERROR
    # A second object gives bit-identical results.
    assert np.array_equal(oracle_lib.hilbert(x), yc)


def test_hilbert_envelope_golden(oracle_lib, golden_vectors):
    """TestMethod::testHilbertTransform (TestMethod.cpp:681-710), envelope part:
    HilbertEnvelope::calculate against test/hilbert_ya.h5."""
    x = golden_vectors["hilbert_x"]
    ya = oracle_lib.envelope(x)
    ref = golden_vectors["hilbert_ya"]
    assert np.abs(ya - ref).max() / np.abs(ref).max() <= HILBERT_MAX_RELATIVE_ABS_ERROR


def test_linear_to_decibels_rules(oracle_lib):
    """Util::linearToDecibels (Util.h:600-613): normalized by the largest
    magnitude, 20 log10, values at or below the floor set to the floor; an
    all-zero input stays at the floor."""
    x = np.array([0.0, 1e-6, 0.5, 2.0, -2.0, 1.0, 1e-3], np.float32)
    y = oracle_lib.linear_to_decibels(x, -40.0)
    assert y[3] == 0.0 and y[4] == -40.0 and y[0] == -40.0 and y[1] == -40.0
    assert abs(y[2] - 20 * np.log10(0.25)) < 1e-5 and abs(y[5] - 20 * np.log10(0.5)) < 1e-5
    assert y[6] == -40.0  # 1e-3 / 2 = 5e-4 < 10^-2
    assert np.all(oracle_lib.linear_to_decibels(np.zeros(5, np.float32), -60.0) == -60.0)


@pytest.mark.parametrize("U", [2, 8, 64])
def test_interpolator_golden(oracle_lib, golden_vectors, U):
    """TestMethod::testInterpolator (TestMethod.cpp:746-794)."""
    x = golden_vectors["interp_source"]
    ref = golden_vectors[f"interp_{U}x"]
    taps = oracle_lib.interp_taps(U, INTERPOLATOR_LP_FILTER_TRANSITION_WIDTH)
    y = oracle_lib.upsample(x, U, taps)
    assert y.size == ref.size
    assert np.abs(y - ref).max() / np.abs(ref).max() <= INTERPOLATOR_MAX_RELATIVE_ABS_ERROR


def test_interpolator4x_golden(oracle_lib, golden_vectors):
    """Interpolator4X against the output the reference's own test saved
    (TestMethod::testInterpolator4X, TestMethod.cpp:796-807): the taps are
    regenerated from the recipe stated in Interpolator4X.h."""
    x, ref = golden_vectors["interp4x_x"], golden_vectors["interp4x_y"]
    y = oracle_lib.upsample(x, 4, oracle_lib.interp4x_taps())
    assert np.abs(y - ref).max() / np.abs(ref).max() <= INTERPOLATOR_MAX_RELATIVE_ABS_ERROR


def test_kaiser_window_golden(oracle_lib, golden_vectors):
    """TestMethod::testKaiserWindow (TestMethod.cpp:809-844), every size entry."""
    tol = golden_vectors["kaiser_tol_db"]
    beta = golden_vectors["kaiser_beta"]
    for t, b in zip(tol, beta):
        if b > 0:
            assert abs(oracle_lib.kaiser_beta(t) - b) / b <= KAISER_MAX_RELATIVE_ABS_ERROR
    for tw in (0.05, 0.1, 0.5):
        ref = golden_vectors[f"kaiser_size_{tw}"]
        got = np.array([oracle_lib.kaiser_size(t, tw) for t in tol])
        assert np.array_equal(got, ref.astype(int))


def test_scf_known_answer(oracle_lib):
    """TestMethod::testSCF (TestMethod.cpp:949-960): exact compare."""
    assert oracle_lib.scf(np.array([1.0, 0.0, -1.0, 1.0, -1.0, 1.0]), 2.0) == 3.270805724762158e-3


@pytest.mark.parametrize("n", [2048, 3571, 4000, 34560 // 2])
def test_fft_against_numpy(oracle_lib, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = oracle_lib.fft(x, -1)
    ref = np.fft.fft(x)
    assert np.abs(y - ref).max() / np.abs(ref).max() <= FFT_MAX_RELATIVE_ABS_ERROR
    yi = oracle_lib.fft(y, +1) / n
    assert np.abs(yi - x).max() <= 1e-12


def test_hilbert_sizes(oracle_lib):
    """HilbertEnvelope padding rule (HilbertEnvelope.h:152)."""
    assert oracle_lib.hilbert_fft_size(4000) == 5120
    assert oracle_lib.hilbert_fft_size(8192) == 9216
    assert oracle_lib.hilbert_fft_size(32768) == 34560
    assert oracle_lib.hilbert_fft_size(4096) == 5120
    assert oracle_lib.hilbert_fft_size(16384) == 17496
    assert oracle_lib.hilbert_fft_size(10) == 2048


def test_remove_dc(oracle_lib):
    rng = np.random.default_rng(3)
    x = rng.standard_normal(1000) + 3.0
    y = oracle_lib.remove_dc(x, 100)
    assert np.allclose(y, x - x[100:].mean(), atol=1e-12)
    with pytest.raises(ValueError):
        oracle_lib.remove_dc(x, 1000)


def _oracle_spec(oracle_lib, d, prefix, **kw):
    from us_lab4a_gb300 import workloads
    from us_lab4a_gb300.config import element_positions_matrix
    if prefix == "vectorial3d_pcf":
        nx = int(d[prefix + "/nx"])
        el = element_positions_matrix(0.3e-3, nx, 0.0, 0.3e-3, nx, 0.0, np.float32)
        tx = rx = el
        fs, fc, U = 24e6, 3e6, 4
    else:
        n = int(d[prefix + "/num_elements"])
        rx = workloads.linear_array(n)
        first = int(d[prefix + "/first_tx"]) if prefix + "/first_tx" in d.files else 0
        last = int(d[prefix + "/last_tx"]) if prefix + "/last_tx" in d.files else n - 1
        tx = rx[first:last + 1]
        fs, fc = 40e6, 5e6
        U = int(d[prefix + "/upsampling"]) if prefix + "/upsampling" in d.files else (1 if prefix == "vectorial_subtx" else 4)
    rf = d[prefix + "/rf"].astype(np.float32)
    return oracle_lib.OracleSpec(tx_xy=tx, rx_xy=rx, num_samples=rf.shape[2], upsampling=U, sampling_frequency=fs,
                                 propagation_speed=1540.0, center_frequency=fc, rx_apod=d[prefix + "/apod"], **kw), rf


FRAME_CASES = {
    "vectorial_plain": dict(cf=0),
    "vectorial_pcf": dict(cf=1, pcf_gamma=1.0, peak_offset=1.5, dead_zone_m=0.5e-3),
    "vectorial_subtx": dict(cf=1, pcf_gamma=2.0),
    "default_scf": dict(cf=2, scf_p=2.0, real_path=True),
    "vectorial3d_pcf": dict(cf=1, pcf_gamma=1.0),
}


@pytest.mark.parametrize("prefix", sorted(FRAME_CASES))
def test_oracle_matches_reference_processor(oracle_lib, golden_frames, prefix):
    """The FP32 oracle reproduces the reference processor's FP32 image within
    1e-5 of the image maximum and its coherence factor within 1e-4."""
    spec, rf = _oracle_spec(oracle_lib, golden_frames, prefix, **FRAME_CASES[prefix])
    grid = golden_frames[prefix + "/grid"]
    v, f, _ = oracle_lib.process(spec, rf, grid, dtype=np.float32)
    vr, fr = golden_frames[prefix + "/value"], golden_frames[prefix + "/factor"]
    assert np.abs(v - vr).max() <= 1e-5 * np.abs(vr).max()
    assert np.abs(f - fr).max() <= 1e-4


def test_oracle_against_compiled_reference_extra_cases(oracle_lib):
    """Direct comparison with the reference processors compiled from their
    sources (only where those were built, i.e. where the reference is present)."""
    from oracle import ref
    if not ref.available():
        pytest.skip("reference processors not built here")
    from us_lab4a_gb300 import workloads
    fr = workloads.cf2d(small=True, seed=77)
    rf = fr.make_rf_numpy()
    n = fr.spec.num_tx
    for cf, extra in ((0, {}), (1, dict(pcf_gamma=0.5))):
        vr, fref = ref.process(rf=rf, grid_xyz=fr.grid_xyz, num_samples=fr.spec.num_samples, upsampling=8,
                               fs=40e6, c=1540.0, fc=5e6, rx_apod=fr.spec.rx_apod, cf=cf, peak_offset=0.7,
                               num_elements=n, first_tx=0, last_tx=n - 1, pitch=0.3e-3, **extra)
        spec = oracle_lib.OracleSpec(tx_xy=fr.spec.tx_xy, rx_xy=fr.spec.rx_xy, num_samples=fr.spec.num_samples,
                                     upsampling=8, sampling_frequency=40e6, propagation_speed=1540.0,
                                     center_frequency=5e6, peak_offset=0.7, rx_apod=fr.spec.rx_apod, cf=cf, **extra)
        v, f, _ = oracle_lib.process(spec, rf, fr.grid_xyz, dtype=np.float32)
        assert np.abs(v - vr).max() <= 1e-5 * np.abs(vr).max()
        assert np.abs(f - fref).max() <= 1e-4


@pytest.mark.parametrize("name", ["synthy_all", "synthy_window_pcf", "t1r1_pcf", "t1r1_plain", "tnrn_diverging",
                                  "tnrn_focused_pcf"])
def test_single_term_oracle_matches_reference_processor(oracle_lib, golden_single, name):
    """The FP32 oracle of the single-term 3D processors reproduces the outputs
    of Vectorial3DT1R1SAFTProcessor / Vectorial3DTnRnProcessor /
    SynthYVectorial3DTnRnProcessor<float> (compiled from the reference's
    sources) within 1e-5 of the image maximum and the coherence factor within
    1e-4; grid points whose every term falls outside the signal are exactly 0
    on both sides."""
    from helpers import single_case
    spec, rf, grid = single_case(oracle_lib, golden_single, name)
    v, f, _ = oracle_lib.single(spec, rf, grid, dtype=np.float32)
    vr, fr = golden_single[name + "/value"], golden_single[name + "/factor"]
    assert np.abs(vr).max() > 0
    assert np.abs(v - vr).max() <= 1e-5 * np.abs(vr).max()
    assert np.abs(f - fr).max() <= 1e-4
    assert np.array_equal(v == 0, vr == 0)


def test_single_term_tx_focus_delays_match_reference(golden_single):
    """ArrayUtil::calculateTx3DFocusDelay restated on the host (focused and
    diverging) gives the reference's delays bit for bit."""
    from us_lab4a_gb300.config import tx_3d_focus_delay
    for name in ("tnrn_focused_pcf", "tnrn_diverging", "synthy_all"):
        g = lambda k: golden_single[name + "/" + k]
        fx, fy, fz = (float(x) for x in g("focus"))
        got = tx_3d_focus_delay(fx, fy, fz, float(g("c")), g("tx_xy"))
        assert np.array_equal(got, g("tx_delays").astype(np.float32)), name


@pytest.mark.parametrize("name", ["onetx_pcf", "onetx_plain", "sta_pcf", "sta_plain"])
def test_two_medium_oracle_matches_reference_processor(oracle_lib, golden_two_medium, name):
    """The FP32 oracle of the two-medium imaging reproduces
    VectorialCombinedTwoMediumImagingProcessor<float> (compiled from the
    reference's sources): Fermat delays, minimum rows, one-transmit and STA
    steps, PCF; within 1e-5 of the image maximum, the same points zero."""
    from helpers import two_medium_case
    spec, rf, grid = two_medium_case(oracle_lib, golden_two_medium, name)
    img = oracle_lib.two_medium(spec, rf, grid, dtype=np.float32)
    ref = golden_two_medium[name + "/image"]
    assert np.abs(ref).max() > 0
    assert np.abs(img - ref).max() <= 1e-5 * np.abs(ref).max()
    assert np.array_equal(img == 0, ref == 0)


def test_two_medium_fermat_block_size_rule(oracle_lib, golden_two_medium):
    """FermatPrinciple::calcBlockSizeForTwoStepSearch takes the maximum block
    size as an unsigned number of wavelengths: 3.5 acts as 3."""
    from helpers import two_medium_case
    spec, rf, grid = two_medium_case(oracle_lib, golden_two_medium, "sta_pcf")
    spec.max_fermat_block_size = 3.0
    a = oracle_lib.two_medium(spec, rf, grid, dtype=np.float32)
    spec.max_fermat_block_size = 3.5
    b = oracle_lib.two_medium(spec, rf, grid, dtype=np.float32)
    assert np.array_equal(a, b)
