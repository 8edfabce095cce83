"""ORACLE (test infrastructure only) -- numpy FP64 model of the GPU pulsar simulator.

Only tests/ import this module, as the checker of msosm_sim_*.  It restates the
generator's algorithm independently of the engine:
  * counter-based normals: Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
    random numbers: as easy as 1, 2, 3", SC'11) on counter (i_lo, i_hi, stream, 0)
    and key (seed_lo, seed_hi), Box-Muller on the top 24 bits of the first two words;
  * emission per pulse kind: the reference generator's three-component test profile
    (simulated_pulsar/simulated_complex_signal.cpp:44-72), one Gaussian component, or
    the two impulses of generate_pulsar_signal (:563-571);
  * dispersion by the causal impulse response built as generate_pulsar_signal_new
    builds it (:347-395: chirp exp(+i phi) at fp = next_pow2(Nd+1) bins, inverse
    transform / fp, taps fp-Nd..fp-1 and 0 moved to 0..Nd), applied as one linear
    convolution by FFT, output sample e = y[e + Nd] (:438-442);
  * additive AWGN at per-sample SNR against the emission's mean power;
  * encodings: complex64, uint16 offset binary (0 = no data), int8 I/Q.
"""
from __future__ import annotations

import numpy as np

KDM = 4.15e15
_MASK = np.uint64(0xFFFFFFFF)
_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)


def philox_rounds(c0, c1, c2, c3, k0: int, k1: int):
    """Philox-4x32-10 of counter words c0..c3 (uint64 arrays of 32-bit values), key (k0, k1)."""
    c0, c1, c2, c3 = (np.asarray(c, np.uint64) for c in (c0, c1, c2, c3))
    k0, k1 = np.uint64(k0), np.uint64(k1)
    for _ in range(10):
        p0 = _M0 * c0
        p1 = _M1 * c2
        c0, c1, c2, c3 = ((p1 >> np.uint64(32)) ^ c1 ^ k0, p1 & _MASK, (p0 >> np.uint64(32)) ^ c3 ^ k1, p0 & _MASK)
        k0 = (k0 + _W0) & _MASK
        k1 = (k1 + _W1) & _MASK
    return c0, c1, c2, c3


def philox4x32_10(idx: np.ndarray, stream: int, seed: int):
    """Four 32-bit words per sample index idx: counter (idx_lo, idx_hi, stream, 0),
    key (seed_lo, seed_hi)."""
    idx = idx.astype(np.uint64)
    c0 = idx & _MASK
    return philox_rounds(c0, idx >> np.uint64(32), np.full_like(c0, np.uint64(stream)), np.zeros_like(c0),
                         seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)


def normal_pairs(idx: np.ndarray, stream: int, seed: int) -> np.ndarray:
    """Complex g = g_re + i g_im of independent N(0, 1) quadratures per counter."""
    r0, r1, _, _ = philox4x32_10(idx, stream, seed)
    # the uniforms are formed in single precision, as on the device
    u1 = ((r0 >> np.uint64(8)).astype(np.float32) + np.float32(0.5)) * np.float32(2.0 ** -24)
    u2 = (r1 >> np.uint64(8)).astype(np.float32) * np.float32(2.0 ** -24)
    rad = np.sqrt(-2.0 * np.log(u1.astype(np.float64)))
    ang = 2.0 * np.pi * u2.astype(np.float64)
    return rad * np.cos(ang) + 1j * rad * np.sin(ang)


def smear(bw: float, dm: float, f0: float) -> int:
    """Nd with the reference's operand types (float kdm*dm, float 1/fs)."""
    bw32, f032, dm32 = np.float32(bw), np.float32(f0), np.float32(dm)
    kd = np.float32(np.float32(4.15e15) * dm32)
    f1 = np.float32(f032 + bw32)
    a = 1.0 / (float(f032) * float(f032))
    b = 1.0 / (float(f1) * float(f1))
    inv_fs = np.float32(np.float32(1.0) / bw32)
    return int(np.floor(float(kd) * (a - b) / float(inv_fs)))


def period_samples(bw: float, period: float) -> int:
    return int(np.float32(np.float32(period) * np.float32(bw)))


def profile(kind: int, Np: int, duty: float = 0.05) -> np.ndarray:
    x = np.arange(Np, dtype=np.float64) / Np
    if kind == 0:
        return (0.45 * np.exp(-0.5 * ((x - 0.455) / 0.008) ** 2) + np.exp(-0.5 * ((x - 0.5) / 0.012) ** 2)
                + 0.28 * np.exp(-0.5 * ((x - 0.555) / 0.006) ** 2))
    sig = duty / (2.0 * np.sqrt(2.0 * np.log(2.0)))
    return np.exp(-0.5 * ((x - 0.5) / sig) ** 2)


def emission(i: np.ndarray, kind: int, Np: int, duty: float, seed: int) -> np.ndarray:
    j = (i % np.uint64(Np)).astype(np.int64)
    if kind == 2:
        return np.where((j == Np // 2) | (j == Np // 2 + 2), 32767.0, 0.0).astype(np.complex128)
    prof = profile(kind, Np, duty)
    amp = prof / prof.max() * 10000.0 / np.sqrt(2.0)
    return amp[j] * normal_pairs(i, 0, seed)


def signal_power(kind: int, Np: int, duty: float) -> float:
    if kind == 2:
        return 2.0 * 32767.0 ** 2 / Np
    prof = profile(kind, Np, duty)
    return float(np.mean((prof / prof.max() * 10000.0) ** 2))


def dispersion_taps(bw: float, f0: float, dm: float, nd: int) -> np.ndarray:
    """Causal impulse response h[0..nd]."""
    fp = 1
    while fp < nd + 1:
        fp <<= 1
    fs = float(np.float32(bw))
    k = np.arange(fp, dtype=np.float64)
    step = fs / fp
    f = np.where(k < fp // 2, fs / 2 + k * step, k * step - fs / 2)
    w = 2 * np.pi * f
    w0 = 2 * np.pi * float(np.float32(f0))
    phase = 4 * np.pi ** 2 * KDM * float(np.float32(dm)) * w * w / ((w + w0) * w0 * w0)
    h = np.fft.ifft(np.exp(1j * phase))  # numpy's ifft includes the 1/fp
    taps = np.empty(nd + 1, np.complex128)
    taps[:nd] = h[fp - nd:]
    taps[nd] = h[0]
    return taps


def generate(n: int, bw: float, f0: float, dm: float, period: float, kind: int = 0, duty: float = 0.05,
             snr_db: float | None = None, seed: int = 1, start: int = 0) -> np.ndarray:
    """Output samples start .. start+n-1 (complex128, before encoding and scale)."""
    Np = period_samples(bw, period)
    nd = smear(bw, dm, f0)
    taps = dispersion_taps(bw, f0, dm, nd)
    # y[t] = sum_k taps[k] x[t - k]; out[e] = y[e + nd] needs x[e .. e + nd]
    i = np.arange(start, start + n + nd, dtype=np.uint64)
    x = emission(i, kind, Np, duty, seed)
    L = 1
    while L < len(x) + nd + 1:
        L <<= 1
    y = np.fft.ifft(np.fft.fft(x, L) * np.fft.fft(taps, L))
    out = y[nd:nd + n]
    if snr_db is not None:
        sigma = np.sqrt(signal_power(kind, Np, duty) / 10 ** (snr_db / 10) / 2)
        out = out + sigma * normal_pairs(np.arange(start, start + n, dtype=np.uint64), 1, seed)
    return out


def encode_u16(v: np.ndarray) -> np.ndarray:
    def enc(c):
        c32 = c.astype(np.float32)
        t = np.clip(c32 + np.float32(32768.0), 0, 65535)
        return np.where(c32 == 0, 0, np.trunc(t)).astype(np.uint32)
    return enc(v.real) | (enc(v.imag) << np.uint32(16))
