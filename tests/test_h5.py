"""Saved acquisitions and images (usgb_h5_*): the library's HDF5 reader against
the reference's own libhdf5-written test files and the golden vectors taken
from them, against chunked files with the shuffle / LZF / deflate filters
built by tests/h5_build.py, the writer by round trip, and the
SavedSTAAcquisition / image-file mirrors. Host code only (no GPU)."""
import os

import numpy as np
import pytest

from oracle.ref import REF_TEST

# golden vector -> reference test file (dataset "v")
PAIRS = {
    "hilbert_x": "hilbert_x.h5", "hilbert_ya": "hilbert_ya.h5", "hilbert_yi": "hilbert_yi.h5",
    "hilbert_yr": "hilbert_yr.h5", "interp_2x": "interp_2x.h5", "interp_64x": "interp_64x.h5",
    "interp_8x": "interp_8x.h5", "interp_source": "interp_source.h5", "kaiser_beta": "kaiser_beta.h5",
    "kaiser_size_0.05": "kaiser_size-trans_width_0.05.h5", "kaiser_size_0.1": "kaiser_size-trans_width_0.1.h5",
    "kaiser_size_0.5": "kaiser_size-trans_width_0.5.h5", "kaiser_tol_db": "kaiser_tol_db.h5",
}


@pytest.fixture(scope="module")
def h5():
    from us_lab4a_gb300 import build
    build.build()
    from us_lab4a_gb300 import h5 as mod
    return mod


@pytest.mark.skipif(not os.path.isdir(REF_TEST), reason="reference test files not present")
def test_reads_reference_libhdf5_files_exactly(h5, golden_vectors):
    """Chunked, deflate-compressed files written by libhdf5 (h5py): every value
    equals the golden vector extracted from the same file."""
    for key, f in PAIRS.items():
        got = h5.read(os.path.join(REF_TEST, f), "v").ravel()
        assert np.array_equal(got, golden_vectors[key].ravel()), key


@pytest.mark.skipif(not os.path.isdir(REF_TEST), reason="reference test files not present")
def test_reads_every_reference_test_file(h5):
    import glob
    n = 0
    for f in sorted(glob.glob(os.path.join(REF_TEST, "*.h5"))):
        for name in ("v", "x", "y", "b", "ascan"):
            try:
                rank, n1, n2 = h5.info(f, name)
            except Exception:
                continue
            a = h5.read(f, name)
            assert a.size == n1 * n2 and np.all(np.isfinite(a))
            n += 1
            break
    assert n >= 30


@pytest.mark.parametrize("shape", [(1, 5), (3, 7), (64, 4096), (1, 1)])
def test_writer_round_trip(h5, tmp_path, shape):
    rng = np.random.default_rng(shape[0] * 31 + shape[1])
    a = rng.standard_normal(shape)
    if a.size > 3:
        a.flat[0], a.flat[1], a.flat[2] = -0.0, np.inf, 1e-310
    p = str(tmp_path / "x.h5")
    h5.write(p, "value", a)
    assert h5.info(p, "value") == (2, shape[0], shape[1])
    b = h5.read(p, "value")
    assert b.shape == shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))
    raw = open(p, "rb").read()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n" and raw[8] == 0
    assert int.from_bytes(raw[40:48], "little") == len(raw)   # end-of-file address


@pytest.mark.parametrize("filters", [("shuffle", "lzf"), ("lzf",), ("shuffle", "deflate"), ("deflate",), ()])
@pytest.mark.parametrize("shape,chunk", [((10, 300), (4, 128)), ((1000,), (256,)), ((3, 5), (3, 5))])
def test_reads_chunked_filtered_files(h5, tmp_path, filters, shape, chunk):
    """Several chunks, edge chunks past the dataset, LZF chunks left
    unfiltered (filter mask) when they do not compress."""
    from h5_build import build_chunked
    rng = np.random.default_rng(7)
    a = np.round(rng.standard_normal(shape) * 8) / 8          # compressible
    if len(shape) == 2:
        a[1] = rng.standard_normal(shape[1])                    # an incompressible row
    p = str(tmp_path / "c.h5")
    open(p, "wb").write(build_chunked("signal", a, chunk, filters))
    b = h5.read(p, "signal")
    assert np.array_equal(b.reshape(a.shape), a)


def test_reads_float32_datasets(h5, tmp_path):
    from h5_build import build_chunked
    a = np.linspace(-1, 1, 500, dtype=np.float32).reshape(5, 100)
    p = str(tmp_path / "f.h5")
    open(p, "wb").write(build_chunked("v", a, (2, 64), ("shuffle", "lzf"), dtype="<f4"))
    assert np.array_equal(h5.read(p, "v"), a.astype(np.float64))


def test_lzf_encoder_matches_decoder_rules(h5, tmp_path):
    """Long matches (length byte), far references, literal runs of 32."""
    from h5_build import build_chunked
    base = np.arange(4096, dtype=np.float64) % 37
    a = np.concatenate([base, base[::-1], np.random.default_rng(1).standard_normal(300)])
    p = str(tmp_path / "l.h5")
    open(p, "wb").write(build_chunked("v", a, (a.size,), ("lzf",)))
    assert np.array_equal(h5.read(p, "v"), a)


def test_errors(h5, tmp_path):
    from us_lab4a_gb300.errors import InvalidParameterException, InvalidValueException
    with pytest.raises(InvalidParameterException, match="Could not open"):
        h5.read(str(tmp_path / "missing.h5"), "v")
    p = str(tmp_path / "x.h5")
    h5.write(p, "value", np.ones((2, 2)))
    with pytest.raises(InvalidParameterException, match="No dataset"):
        h5.read(p, "signal")
    q = str(tmp_path / "bad.h5")
    open(q, "wb").write(b"not an hdf5 file at all" * 10)
    with pytest.raises(InvalidValueException, match="not an HDF5 file"):
        h5.read(q, "v")
    open(q, "wb").write(open(p, "rb").read()[:200])
    with pytest.raises(InvalidValueException):
        h5.read(q, "value")
    with pytest.raises(InvalidParameterException, match="equal to 0"):
        h5.write(p, "value", np.ones((0, 3)))


def test_saved_acquisition_and_image_files(h5, tmp_path):
    """SavedSTAAcquisition reads signals-base####-tx####.h5 "signal" (num_rx
    rows); images go to image_value / image_factor / image_x,y,z.h5."""
    from us_lab4a_gb300 import InvalidValueException, make_grid
    rng = np.random.default_rng(3)
    rf = rng.standard_normal((3, 8, 100)).astype(np.float32)
    d = str(tmp_path / "acq")
    for tx in range(3):
        h5.save_tx_elem_signals(rf[tx], d, 16, tx)
    assert os.path.exists(os.path.join(d, "signals-base0016-tx0002.h5"))
    acq = h5.SavedSTAAcquisition(8, d)
    acq.prepare(16)
    for tx in range(3):
        assert np.array_equal(acq.execute(tx), rf[tx])
    wrong = h5.SavedSTAAcquisition(7, d)
    wrong.prepare(16)
    with pytest.raises(InvalidValueException, match="Invalid number of rx elements"):
        wrong.execute(0)
    grid = make_grid(4, 6)
    grid["x"] = rng.standard_normal((4, 6))
    grid["z"] = rng.standard_normal((4, 6))
    grid["value"] = rng.standard_normal((4, 6))
    grid["factor"] = rng.uniform(0, 1, (4, 6))
    out = str(tmp_path / "img")
    h5.save_image(grid, out)
    v, f = h5.load_image(out)
    assert np.array_equal(v, grid["value"].astype(np.float64)) and np.array_equal(f, grid["factor"].astype(np.float64))
    assert np.array_equal(h5.read(os.path.join(out, "image_z.h5"), "z"), grid["z"].astype(np.float64))

