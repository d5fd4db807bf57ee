"""Regenerates the golden fixtures of tests/golden/ (run where the reference
sources are present; the fixtures are committed and travel with the tests).

1. reference_vectors.npz: the reference's own golden vectors from its test
   directory (test/*.h5; written by test/gen_*.py with scipy and by
   TestMethod::testInterpolator4X): Hilbert input/outputs, interpolation 2x/8x/64x,
   Interpolator4X input/output, Kaiser beta/size tables. The files are
   chunked, deflate-compressed HDF5 1-D float64 datasets; each chunk is one
   zlib stream, stored in dataset order, so the data is recovered by
   inflating every zlib stream in file order (lengths are checked against
   the shapes the reference's tests expect).
2. reference_frames.npz: outputs of the reference processors themselves
   (VectorialSTAProcessor, Vectorial3DSTAProcessor, DefaultSTAProcessor,
   compiled from their sources by oracle/refbuild) on small seeded frames,
   with the inputs (RF, grid, parameters) stored beside them.
3. reference_single.npz: the same for the single-term 3D processors
   (Vectorial3DT1R1SAFTProcessor, Vectorial3DTnRnProcessor,
   SynthYVectorial3DTnRnProcessor) on a 6 x 5 matrix array, every input
   parameter stored beside the outputs.
4. reference_windows.npz: the reference's WindowFunction::get<float> for every
   window name at sizes 2..256 and for trapezoidal descriptions (the
   apodization vectors of the processors).
5. reference_two_medium.npz: the same for VectorialCombinedTwoMediumImagingProcessor
   (one transmit element per step and STA steps, with and without PCF) on
   small two-medium scenes (noise-free RF, stored as FP16 values).

Usage: python tests/golden/make_golden.py [--reference <reference root>]
           [--vectors-only | --single-only | --two-medium-only | --windows-only]
"""
from __future__ import annotations

import argparse
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def h5_float64(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    out = []
    i = 0
    while i < len(data) - 2:
        if data[i] == 0x78 and ((data[i] << 8) | data[i + 1]) % 31 == 0:
            d = zlib.decompressobj()
            try:
                r = d.decompress(data[i:])
            except zlib.error:
                i += 1
                continue
            if d.eof and r and len(r) % 8 == 0:
                out.append(np.frombuffer(r, "<f8"))
                i = len(data) - len(d.unused_data)
                continue
        i += 1
    if not out:
        raise RuntimeError(f"no data in {path}")
    return np.concatenate(out)


def reference_vectors(ref_test: str) -> dict:
    r = lambda n: h5_float64(os.path.join(ref_test, n + ".h5"))  # noqa: E731
    v = {
        "hilbert_x": r("hilbert_x"), "hilbert_yr": r("hilbert_yr"), "hilbert_yi": r("hilbert_yi"),
        "hilbert_ya": r("hilbert_ya"),
        "interp_source": r("interp_source"),
        "interp_2x": r("interp_2x"), "interp_8x": r("interp_8x"), "interp_64x": r("interp_64x"),
        "interp4x_x": r("interp_x"), "interp4x_y": r("interp_y"),
        "kaiser_tol_db": r("kaiser_tol_db"), "kaiser_beta": r("kaiser_beta"),
        "kaiser_size_0.05": r("kaiser_size-trans_width_0.05"), "kaiser_size_0.1": r("kaiser_size-trans_width_0.1"),
        "kaiser_size_0.5": r("kaiser_size-trans_width_0.5"),
    }
    n = v["hilbert_x"].size
    assert v["hilbert_yr"].size == n and v["hilbert_yi"].size == n and v["hilbert_ya"].size == n
    m = v["interp_source"].size
    for U in (2, 8, 64):
        assert v[f"interp_{U}x"].size == m * U, (U, v[f"interp_{U}x"].size)
    assert v["interp4x_y"].size == 4 * v["interp4x_x"].size
    assert v["kaiser_beta"].size == v["kaiser_tol_db"].size
    return v


def _quantized(fr):
    """RF rounded to FP16 values (exact float32 inputs; halves the fixture size)."""
    fr.rf = fr.make_rf_numpy().astype(np.float16).astype(np.float32)
    return fr


def reference_frames() -> dict:
    from oracle import ref
    from us_lab4a_gb300 import workloads
    out = {}

    def put(prefix, fr, value, factor, **meta):
        out[prefix + "/rf"] = fr.make_rf_numpy().astype(np.float16)
        out[prefix + "/grid"] = fr.grid_xyz
        out[prefix + "/apod"] = np.asarray(fr.spec.rx_apod if fr.spec.rx_apod is not None else np.ones(fr.spec.num_rx), np.float32)
        out[prefix + "/value"] = value
        out[prefix + "/factor"] = factor
        for k, x in meta.items():
            out[prefix + "/" + k] = np.asarray(x)

    # VectorialSTAProcessor<float>, no CF.
    fr = _quantized(workloads.plain2d(tiny=True))
    n = fr.spec.num_tx
    kw = dict(num_samples=fr.spec.num_samples, upsampling=fr.spec.upsampling, fs=fr.spec.sampling_frequency,
              c=fr.spec.propagation_speed, fc=fr.spec.center_frequency, rx_apod=fr.spec.rx_apod,
              num_elements=n, first_tx=0, last_tx=n - 1, pitch=0.3e-3)
    v, f = ref.process(rf=fr.make_rf_numpy(), grid_xyz=fr.grid_xyz, cf=0, **kw)
    put("vectorial_plain", fr, v, f, num_elements=n, upsampling=fr.spec.upsampling, cf=0)
    # VectorialSTAProcessor<float> with PCF, a peak offset and a dead zone.
    fr = _quantized(workloads.cf2d(tiny=True))
    n = fr.spec.num_tx
    kw = dict(num_samples=fr.spec.num_samples, upsampling=fr.spec.upsampling, fs=fr.spec.sampling_frequency,
              c=fr.spec.propagation_speed, fc=fr.spec.center_frequency, rx_apod=fr.spec.rx_apod,
              num_elements=n, first_tx=0, last_tx=n - 1, pitch=0.3e-3)
    v, f = ref.process(rf=fr.make_rf_numpy(), grid_xyz=fr.grid_xyz, cf=1, pcf_gamma=1.0, peak_offset=1.5,
                       dead_zone_m=0.5e-3, **kw)
    put("vectorial_pcf", fr, v, f, num_elements=n, upsampling=fr.spec.upsampling, cf=1, pcf_gamma=1.0,
        peak_offset=1.5, dead_zone_m=0.5e-3)
    # Sub-aperture transmit (first_tx_elem..last_tx_elem), U = 1 (no interpolation).
    fr = _quantized(workloads.plain2d(tiny=True, seed=1010))
    n = fr.spec.num_tx
    rf = fr.make_rf_numpy()[3:9]
    kw = dict(num_samples=fr.spec.num_samples, upsampling=1, fs=fr.spec.sampling_frequency,
              c=fr.spec.propagation_speed, fc=fr.spec.center_frequency, rx_apod=fr.spec.rx_apod,
              num_elements=n, first_tx=3, last_tx=8, pitch=0.3e-3)
    v, f = ref.process(rf=rf, grid_xyz=fr.grid_xyz, cf=1, pcf_gamma=2.0, **kw)
    out["vectorial_subtx/rf"] = rf.astype(np.float16)
    out["vectorial_subtx/grid"] = fr.grid_xyz
    out["vectorial_subtx/apod"] = np.asarray(fr.spec.rx_apod, np.float32)
    out["vectorial_subtx/value"] = v
    out["vectorial_subtx/factor"] = f
    out["vectorial_subtx/first_tx"] = np.asarray(3)
    out["vectorial_subtx/last_tx"] = np.asarray(8)
    out["vectorial_subtx/num_elements"] = np.asarray(n)
    out["vectorial_subtx/pcf_gamma"] = np.asarray(2.0)
    # DefaultSTAProcessor<float> (real RF, fixed 4x FIR) with SCF p = 2.
    fr = _quantized(workloads.plain2d(tiny=True, seed=1011))
    n = fr.spec.num_tx
    v, f = ref.process(rf=fr.make_rf_numpy(), grid_xyz=fr.grid_xyz, num_samples=fr.spec.num_samples, upsampling=4,
                       fs=fr.spec.sampling_frequency, c=fr.spec.propagation_speed, fc=fr.spec.center_frequency,
                       cf=2, scf_p=2.0, real_path=True, num_elements=n, first_tx=0, last_tx=n - 1, pitch=0.3e-3)
    put("default_scf", fr, v, f, num_elements=n, cf=2, scf_p=2.0)
    # Vectorial3DSTAProcessor<float> with PCF (6 x 6 matrix array).
    fr = _quantized(workloads.matrix3d(tiny=True))
    v, f = ref.process(rf=fr.make_rf_numpy(), grid_xyz=fr.grid_xyz, num_samples=fr.spec.num_samples, upsampling=4,
                       fs=fr.spec.sampling_frequency, c=fr.spec.propagation_speed, fc=fr.spec.center_frequency,
                       rx_apod=fr.spec.rx_apod, cf=1, pcf_gamma=1.0, matrix=(4, 4, 0.3e-3, 0.3e-3))
    put("vectorial3d_pcf", fr, v, f, nx=4, cf=1, pcf_gamma=1.0)
    return out


SINGLE_ARRAY = (6, 5, 0.3e-3, 0.3e-3)   # nx, ny, pitch_x, pitch_y
SINGLE_ACQ_Y = (-0.6e-3, -0.3e-3, 0.0, 0.3e-3, 0.6e-3)

# name: (mode, parameters). T1R1: active elements; TnRn: base element, group
# size, focus z; synthetic y: window of the five acquisitions.
SINGLE_CASES = {
    "t1r1_plain": (0, dict(active=(0, 2, 3, 5, 7, 11, 13, 17, 20, 29), upsampling=4, cf=0, peak_offset=1.5,
                           dead_zone_m=1e-3)),
    "t1r1_pcf": (0, dict(active=tuple(range(30)), upsampling=8, cf=1, pcf_gamma=1.0, peak_offset=1.0)),
    "tnrn_focused_pcf": (1, dict(base_element=3, num_elements=20, focus_z=4e-3, upsampling=4, cf=1, pcf_gamma=1.0,
                                 peak_offset=1.5, dead_zone_m=1e-3, apod="hann")),
    "tnrn_diverging": (1, dict(base_element=0, num_elements=30, focus_z=-5e-3, upsampling=1, cf=0, peak_offset=0.5)),
    "synthy_window_pcf": (2, dict(base_element=0, num_elements=30, focus_z=-3e-3, upsampling=4, cf=1, pcf_gamma=2.0,
                                  peak_offset=1.5, first_acq=1, last_acq=3)),
    "synthy_all": (2, dict(base_element=0, num_elements=30, focus_z=-3e-3, upsampling=4, cf=0, peak_offset=1.5,
                           first_acq=0, last_acq=4, apod="hann")),
}


def reference_single_frames() -> dict:
    from oracle import ref
    from us_lab4a_gb300 import synth
    from us_lab4a_gb300.config import element_positions_matrix
    from us_lab4a_gb300.workloads import grid_xyz3
    fs, c, fc, ns = 40e6, 1540.0, 5e6, 400
    nx, ny, pitch_x, pitch_y = SINGLE_ARRAY
    el = element_positions_matrix(pitch_x, nx, 0.0, pitch_y, ny, 0.0, np.float32)
    grid = grid_xyz3(-2e-3, 2e-3, 5, -1e-3, 1e-3, 3, 3e-3, 7e-3, 32).astype(np.float32).reshape(15, 32, 3)
    out = {}
    for i, (name, (mode, p)) in enumerate(sorted(SINGLE_CASES.items())):
        rng = np.random.default_rng(2000 + i)
        scat = synth.point_scatterers(rng, 6, (-2e-3, 2e-3), (3.5e-3, 6.5e-3), y_range=(-1e-3, 1e-3))
        kw = dict(grid_xyz=grid, matrix=SINGLE_ARRAY, num_samples=ns, upsampling=p["upsampling"], fs=fs, c=c, fc=fc,
                  peak_offset=p.get("peak_offset", 0.0), dead_zone_m=p.get("dead_zone_m", 0.0), cf=p["cf"],
                  pcf_gamma=p.get("pcf_gamma", 1.0), dtype=np.float32)
        meta = dict(mode=mode, num_samples=ns, upsampling=p["upsampling"], fs=fs, c=c, fc=fc,
                    peak_offset=kw["peak_offset"], dead_zone_m=kw["dead_zone_m"], cf=p["cf"],
                    pcf_gamma=kw["pcf_gamma"], grid=grid)
        if mode == 0:
            act = np.asarray(p["active"], np.uint32)
            full = synth.synth_rf_numpy(el[act], el[act], scat, fs, c, fc, ns, rng)
            rf = np.stack([full[k, k] for k in range(act.size)]).astype(np.float16).astype(np.float32)
            v, f, _ = ref.single(mode=0, rf=rf, active=act, **kw)
            meta.update(tx_xy=el[act], rx_xy=el[act], active=act)
        else:
            b, n = p["base_element"], p["num_elements"]
            grp = el[b:b + n]
            focus = (float(np.float32(grp[:, 0].mean())), float(np.float32(grp[:, 1].mean())), p["focus_z"])
            apod = (np.hanning(n + 2)[1:-1] if p.get("apod") == "hann" else np.ones(n)).astype(np.float32)
            src = np.array([[focus[0], focus[1]]])
            if mode == 1:
                rf = synth.synth_rf_numpy(src, grp, scat, fs, c, fc, ns, rng)[0]
                rf = rf.astype(np.float16).astype(np.float32)
                v, f, txd = ref.single(mode=1, rf=rf, base_element=b, num_elements=n, rx_apod=apod, focus=focus, **kw)
            else:
                ys = np.asarray(SINGLE_ACQ_Y, np.float32)
                rf = np.stack([synth.synth_rf_numpy(src, grp + np.array([0.0, y], np.float32), scat, fs, c, fc, ns, rng)[0]
                               for y in ys]).astype(np.float16).astype(np.float32)
                v, f, txd = ref.single(mode=2, rf=rf, base_element=b, num_elements=n, rx_apod=apod, focus=focus,
                                       acq_y=ys, first_acq=p["first_acq"], last_acq=p["last_acq"], **kw)
                meta.update(acq_y=ys, first_acq=p["first_acq"], last_acq=p["last_acq"])
            meta.update(tx_xy=grp, rx_xy=grp, rx_apod=apod, focus=np.asarray(focus, np.float32), tx_delays=txd,
                        base_element=b)
        meta.update(rf=rf.astype(np.float16), value=v, factor=f)
        for k, x in meta.items():
            out[name + "/" + k] = np.asarray(x)
    return out


# name: (one transmit element per step, steps, upsampling, CF, PCF gamma, max Fermat block size)
TWO_MEDIUM_CASES = {
    "onetx_plain": (True, 4, 4, 0, 1.0, 2.0),
    "onetx_pcf": (True, 3, 4, 1, 1.0, 2.0),
    "sta_plain": (False, 3, 2, 0, 1.0, 2.0),
    "sta_pcf": (False, 3, 4, 1, 2.0, 3.5),
}


def two_medium_spec(oracle_mod, sc, cf, gamma):
    return oracle_mod.TwoMediumSpec(
        num_elements=sc.num_elements, num_elements_mux=sc.num_elements_mux, pitch=sc.pitch,
        center_frequency=sc.center_frequency, propagation_speed_1=sc.propagation_speed_1,
        propagation_speed_2=sc.propagation_speed_2, sampling_frequency=sc.sampling_frequency,
        num_samples=sc.num_samples, upsampling=sc.upsampling, steps=sc.steps, interface_xz=sc.interface_xz,
        rx_apod=sc.rx_apod, max_fermat_block_size=sc.max_fermat_block_size, peak_offset=sc.peak_offset,
        signal_start_offset=sc.signal_start_offset, cf=cf, pcf_gamma=gamma)


def reference_two_medium_frames() -> dict:
    import oracle
    from oracle import ref
    from us_lab4a_gb300 import workloads
    out = {}
    for i, (name, (one_tx, nsteps, U, cf, gamma, mfbs)) in enumerate(sorted(TWO_MEDIUM_CASES.items())):
        sc = workloads.two_medium_scene(one_tx, num_elements=8, num_elements_mux=16, num_steps=nsteps,
                                        num_samples=1000, upsampling=U, grid=(24, 64), tx_element=3,
                                        sampling_frequency=20e6, num_scatterers=8, noise_std=0.0, seed=3000 + i)
        sc.rf = sc.rf.astype(np.float16).astype(np.float32)
        sc.max_fermat_block_size = mfbs
        img = ref.two_medium(two_medium_spec(oracle, sc, cf, gamma), sc.rf, sc.grid_xz, dtype=np.float32)
        meta = dict(num_elements=sc.num_elements, num_elements_mux=sc.num_elements_mux, pitch=sc.pitch,
                    fc=sc.center_frequency, c1=sc.propagation_speed_1, c2=sc.propagation_speed_2,
                    fs=sc.sampling_frequency, upsampling=U, steps=sc.steps, interface_xz=sc.interface_xz,
                    rx_apod=sc.rx_apod, grid_xz=sc.grid_xz, rf=sc.rf.astype(np.float16), max_fermat_block_size=mfbs,
                    peak_offset=sc.peak_offset, signal_start_offset=sc.signal_start_offset, cf=cf, pcf_gamma=gamma,
                    image=img)
        for k, x in meta.items():
            out[name + "/" + k] = np.asarray(x)
    return out


WINDOW_NAMES = ("rectangular", "triangular", "triangular2", "hanning", "hanning2", "hamming", "blackman",
                "blackman2")
WINDOW_SIZES = (2, 3, 4, 7, 8, 15, 16, 31, 32, 63, 64, 96, 127, 128, 256)
TRAPEZOIDAL = (("trapezoidal", (1, 0, 1)), ("trapezoidal", (3, 4, 5)), ("trapezoidal", (8, 16, 8)),
               ("trapezoidal", (0, 10, 6)), ("trapezoidal2", (3, 4, 5)), ("trapezoidal2", (16, 32, 16)),
               ("trapezoidal2", (5, 0, 0)))


def reference_windows() -> dict:
    """reference_windows.npz: the reference's WindowFunction::get<float> for
    every window name at the array sizes the processors use (and odd ones),
    and the trapezoidal forms, from the compiled reference."""
    from oracle import ref
    out = {}
    for name in WINDOW_NAMES:
        for n in WINDOW_SIZES:
            out[f"{name}/{n}"] = ref.window(name, n)
    for name, (a, b, c) in TRAPEZOIDAL:
        out[f"{name} {a} {b} {c}/{a + b + c}"] = ref.window(f"{name} {a} {b} {c}", a + b + c)
    return out


def main():
    ap = argparse.ArgumentParser()
    from oracle.ref import REF_ROOT
    ap.add_argument("--reference", default=REF_ROOT, help="reference project root (default: US_LAB4A_REFERENCE)")
    ap.add_argument("--vectors-only", action="store_true", help="rewrite reference_vectors.npz only")
    ap.add_argument("--single-only", action="store_true", help="rewrite reference_single.npz only")
    ap.add_argument("--two-medium-only", action="store_true", help="rewrite reference_two_medium.npz only")
    ap.add_argument("--windows-only", action="store_true", help="rewrite reference_windows.npz only")
    args = ap.parse_args()
    if args.windows_only:
        from oracle import ref
        if not ref.available():
            ref.build()
        np.savez_compressed(os.path.join(HERE, "reference_windows.npz"), **reference_windows())
        print("reference_windows.npz", os.path.getsize(os.path.join(HERE, "reference_windows.npz")))
        return
    if args.two_medium_only:
        from oracle import ref
        if not ref.available():
            ref.build()
        np.savez_compressed(os.path.join(HERE, "reference_two_medium.npz"), **reference_two_medium_frames())
        print("reference_two_medium.npz", os.path.getsize(os.path.join(HERE, "reference_two_medium.npz")))
        return
    if args.single_only:
        from oracle import ref
        if not ref.available():
            ref.build()
        np.savez_compressed(os.path.join(HERE, "reference_single.npz"), **reference_single_frames())
        print("reference_single.npz", os.path.getsize(os.path.join(HERE, "reference_single.npz")))
        return
    vec = reference_vectors(os.path.join(args.reference, "test"))
    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"), **vec)
    if args.vectors_only:
        print("reference_vectors.npz", os.path.getsize(os.path.join(HERE, "reference_vectors.npz")))
        return
    from oracle import ref
    if not ref.available():
        ref.build()
    frames = reference_frames()
    np.savez_compressed(os.path.join(HERE, "reference_frames.npz"), **frames)
    np.savez_compressed(os.path.join(HERE, "reference_single.npz"), **reference_single_frames())
    np.savez_compressed(os.path.join(HERE, "reference_two_medium.npz"), **reference_two_medium_frames())
    np.savez_compressed(os.path.join(HERE, "reference_windows.npz"), **reference_windows())
    for f in ("reference_vectors.npz", "reference_frames.npz", "reference_single.npz", "reference_two_medium.npz",
              "reference_windows.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
