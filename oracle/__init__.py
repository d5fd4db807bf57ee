"""CPU oracle for the STA/TFM delay-and-sum path (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package, as the checker. The product (``us_lab4a_gb300``) never imports it.
"""
from .oracle import (  # noqa: F401
    OracleSpec, available, build, lib_path, process, das, interp_taps, interp4x_taps,
    upsample, hilbert, envelope, linear_to_decibels, fft, remove_dc, scf, pcf, hilbert_fft_size,
    next_fast_even_size,
    kaiser_beta, kaiser_size,
    SingleSpec, single, SINGLE_T1R1_SAFT, SINGLE_TNRN, SINGLE_SYNTH_Y_TNRN,
    TwoMediumSpec, two_medium,
)
