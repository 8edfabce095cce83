"""Synthetic dispersed-pulsar baseband (the simulated_pulsar front end).

Restates the signal model of the reference's generator
(simulated_pulsar/simulated_complex_signal.cpp:44-72 pulse, :279-467 dispersion
by one long transform, simulated_pulsar/AWGN.cpp:29-58 noise) with numpy and a
seeded generator:

  * emission: complex Gaussian noise shaped by a Gaussian pulse profile
    (FWHM = duty * period, centred at phase 0.5), one realisation per period
    template, repeated every period;
  * dispersion: the template is multiplied in the frequency domain by
    exp(+i phi(f)), phi = 4 pi^2 kdm DM w^2 / ((w + w0) w0^2), w = 2 pi (f - f0),
    the conjugate of the response the processor removes; bins are mapped to
    w exactly as the reference's dispersion transfer function
    (simulated_complex_signal.cpp:186-204);
  * noise: complex AWGN at the given per-sample SNR (average signal power over
    a period / noise power).

The dispersed template is computed once (one transform of the next power of two
above period + Nd samples) and tiled, so long streams cost a few seconds.
"""
from __future__ import annotations

import numpy as np

KDM = 4.15e15


def smear_samples(bw: float, dm: float, f0: float) -> int:
    f0 = float(np.float32(f0))
    bw = float(np.float32(bw))
    return int(np.floor(KDM * dm * (1 / f0 ** 2 - 1 / (f0 + bw) ** 2) * bw))


def dispersion_phase(nfft: int, bw: float, f0: float, dm: float) -> np.ndarray:
    """phi for FFT bins in numpy order: bin k < nfft/2 sits at f0 + bw/2 + k*bw/nfft."""
    k = np.arange(nfft, dtype=np.float64)
    step = bw / nfft
    f_off = np.where(k < nfft // 2, bw / 2 + k * step, k * step - bw / 2)
    w = 2 * np.pi * f_off
    w0 = 2 * np.pi * f0
    return 4 * np.pi ** 2 * KDM * dm * w * w / ((w + w0) * w0 * w0)


def pulsar_signal(n: int, bw: float, f0: float, dm: float, period: float, duty: float = 0.05,
                  snr_db: float = -10.0, seed: int = 1, dtype=np.complex64) -> np.ndarray:
    """n complex samples at fs = bw of a dispersed pulse train plus AWGN."""
    rng = np.random.default_rng(seed)
    fs = float(bw)
    Np = int(round(period * fs))
    nd = smear_samples(bw, dm, f0)
    # one period of emission: profile * complex Gaussian noise
    x = (np.arange(Np) + 0.5) / Np
    sigma = duty / (2 * np.sqrt(2 * np.log(2)))
    prof = np.exp(-0.5 * ((x - 0.5) / sigma) ** 2)
    emit = prof * (rng.standard_normal(Np) + 1j * rng.standard_normal(Np)) / np.sqrt(2)
    # disperse once; the template is as long as period + smear
    L = 1
    while L < Np + nd + 1:
        L <<= 1
    spec = np.fft.fft(emit, L)
    spec *= np.exp(1j * dispersion_phase(L, fs, float(f0), dm))
    tmpl = np.fft.ifft(spec)
    # tile: period k starts at k*Np; templates extending past n are cut
    sig = np.zeros(n + L, dtype=np.complex128)
    first = -((L + Np - 1) // Np)
    for k in range(first, n // Np + 1):
        s = k * Np
        a, b = max(s, 0), min(s + L, n)
        if a < b:
            sig[a:b] += tmpl[a - s:b - s]
    sig = sig[:n]
    p_sig = np.mean(np.abs(tmpl[:L]) ** 2) * L / Np  # average power per sample over a period
    p_noise = p_sig / (10 ** (snr_db / 10))
    noise = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.sqrt(p_noise / 2)
    return (sig + noise).astype(dtype)


def to_u16(x: np.ndarray, scale: float) -> np.ndarray:
    """Offset-binary uint16 pairs packed in uint32 (low = re, high = im), as the
    reference's simulator writes them (simulated_complex_signal.cpp:258-263)."""
    re = np.clip(np.round(x.real * scale) + 32768, 1, 65535).astype(np.uint32)
    im = np.clip(np.round(x.imag * scale) + 32768, 1, 65535).astype(np.uint32)
    return (im << 16) | re


def to_i8(x: np.ndarray, scale: float) -> np.ndarray:
    """int8 interleaved I/Q, clipped to [-127, 127]."""
    out = np.empty(2 * x.size, np.int8)
    out[0::2] = np.clip(np.round(x.real * scale), -127, 127)
    out[1::2] = np.clip(np.round(x.imag * scale), -127, 127)
    return out
