"""Shared helpers of the parity tests: mapping a workload frame to the oracle,
running it through the library, and error metrics."""
from __future__ import annotations

import numpy as np

CF_CODE = {"none": 0, "pcf": 1, "scf": 2, "mf": 3}


def oracle_spec(oracle_lib, spec, nthreads=None):
    kw = {}
    if nthreads:
        kw["nthreads"] = nthreads
    return oracle_lib.OracleSpec(
        tx_xy=spec.tx_xy, rx_xy=spec.rx_xy, num_samples=spec.num_samples,
        upsampling=4 if spec.real_path else spec.upsampling, sampling_frequency=spec.sampling_frequency,
        propagation_speed=spec.propagation_speed, center_frequency=spec.center_frequency,
        peak_offset=spec.peak_offset, dead_zone_m=spec.dead_zone_m,
        rx_apod=spec.rx_apod if spec.rx_apod is not None else np.ones(spec.num_rx, np.float32),
        cf=CF_CODE[spec.coherence], pcf_gamma=spec.pcf_gamma, scf_p=spec.scf_p, real_path=spec.real_path, **kw)


def run_host(spec, rf, grid_xyz):
    """Through the host C-ABI path (submit_rf + process)."""
    from us_lab4a_gb300 import StaEngine
    with StaEngine(spec) as eng:
        eng.set_grid(grid_xyz)
        return eng.process_host(rf)


def run_device(spec, rf, grid_xyz, device="cuda:0", variant=None):
    """Through the device C-ABI path (resident torch tensors)."""
    import torch
    from us_lab4a_gb300 import StaEngine
    with StaEngine(spec) as eng:
        if variant is not None:
            eng.set_das_variant(variant)
        stream = torch.cuda.current_stream()
        eng.set_stream(stream)
        g = torch.as_tensor(np.ascontiguousarray(grid_xyz, np.float32), device=device)
        r = torch.as_tensor(np.ascontiguousarray(rf, np.float32), device=device)
        v = torch.empty(grid_xyz.shape[:2], dtype=torch.float32, device=device)
        f = torch.empty_like(v)
        eng.set_grid_device(g)
        eng.process_device(r, v, f)
        eng.synchronize()
        return v.cpu().numpy(), f.cpu().numpy()


def rel_err(a, b) -> float:
    """max |a - b| / max |b|, for real or complex images."""
    a, b = np.asarray(a), np.asarray(b)
    t = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    return float(np.abs(a.astype(t) - b.astype(t)).max() / np.abs(b.astype(t)).max())


def db_err(a, b) -> float:
    """Peak-relative error in dB: 20 log10(max |a - b| / max |b|)."""
    e = rel_err(a, b)
    return -np.inf if e == 0 else 20.0 * np.log10(e)


SINGLE_CASE_NAMES = ("synthy_all", "synthy_window_pcf", "t1r1_pcf", "t1r1_plain", "tnrn_diverging", "tnrn_focused_pcf")


def single_case(oracle_lib, d, name):
    """(SingleSpec, rf (acquisitions of the window) float32, grid) of one case
    of reference_single.npz."""
    g = lambda k: d[name + "/" + k]
    mode = int(g("mode"))
    rf = g("rf").astype(np.float32)
    kw = {}
    if mode != 0:
        kw = dict(rx_apod=g("rx_apod"), focus=tuple(float(x) for x in g("focus")), first_tx_delay=float(g("tx_delays")[0]))
    if mode == 2:
        a, b = int(g("first_acq")), int(g("last_acq"))
        kw["acq_y"] = g("acq_y")[a:b + 1]
        rf = rf[a:b + 1]
    spec = oracle_lib.SingleSpec(mode=mode, tx_xy=g("tx_xy"), rx_xy=g("rx_xy"), num_samples=int(g("num_samples")),
                                 upsampling=int(g("upsampling")), sampling_frequency=float(g("fs")),
                                 propagation_speed=float(g("c")), center_frequency=float(g("fc")),
                                 peak_offset=float(g("peak_offset")), dead_zone_m=float(g("dead_zone_m")),
                                 cf=int(g("cf")), pcf_gamma=float(g("pcf_gamma")), **kw)
    return spec, rf, g("grid")


TWO_MEDIUM_CASE_NAMES = ("onetx_pcf", "onetx_plain", "sta_pcf", "sta_plain")


def two_medium_case(oracle_lib, d, name):
    """(TwoMediumSpec, rf float32 (num_acq, num_tx, num_elements, num_samples), grid_xz)
    of one case of reference_two_medium.npz."""
    g = lambda k: d[name + "/" + k]
    rf = g("rf").astype(np.float32)
    spec = oracle_lib.TwoMediumSpec(
        num_elements=int(g("num_elements")), num_elements_mux=int(g("num_elements_mux")), pitch=float(g("pitch")),
        center_frequency=float(g("fc")), propagation_speed_1=float(g("c1")), propagation_speed_2=float(g("c2")),
        sampling_frequency=float(g("fs")), num_samples=rf.shape[3], upsampling=int(g("upsampling")),
        steps=g("steps"), interface_xz=g("interface_xz"), rx_apod=g("rx_apod"),
        max_fermat_block_size=float(g("max_fermat_block_size")), peak_offset=float(g("peak_offset")),
        signal_start_offset=int(g("signal_start_offset")), cf=int(g("cf")), pcf_gamma=float(g("pcf_gamma")))
    return spec, rf, g("grid_xz")
