"""ORACLE (test infrastructure only) -- ctypes binding of oracle/lib/libmsosm_oracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
import this module, and only as the checker or the timed CPU baseline.  The
product never imports it.

The functions restate the reference (joezhouchenye/AcceleratedMS-OSM):
  plan()        Prepare_MSOSM ctor + calculate_min_order + initialize_uint16's
                choice of M + segmentation + generate_dedisp_params
                (dedispersion/msosm/msosm_prepare.cpp:3-284,
                 dedispersion/msosm/msosm_gpu_batch.cpp:32-44,54-61,86-93,113-117)
  Msosm         the streaming processor (msosm_gpu_batch.cpp:153-236 with the
                kernels of gpu/gpu_kernel.cu), FP64 or FP32
  fold()        foldDataPhase (gpu/gpu_kernel.cu:462-485)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "lib" / "libmsosm_oracle.so"
REF_LIB_PATH = HERE / "_ref" / "libmsosm_ref.so"
REF_SEG_LIB_PATH = HERE / "_ref" / "libmsosm_ref_seg.so"
# the reference source tree, for building oracle/_ref; only where it is given
REFERENCE_ROOT_ENV = "MSOSM_REFERENCE_ROOT"

_lib = None


def build(quiet: bool = True) -> Path:
    """Compile the C restatement (gcc; a second or two)."""
    out = subprocess.run(["make", "-C", str(HERE), "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def build_ref(ref_root: str | None = None) -> Path | None:
    """Compile the reference's own planning sources and build_segments (only where the
    tree is given, as an argument or through MSOSM_REFERENCE_ROOT)."""
    ref_root = ref_root or os.environ.get(REFERENCE_ROOT_ENV)
    if not ref_root or not Path(ref_root).is_dir():
        return None
    out = subprocess.run(["make", "-C", str(HERE), "ref", f"REF_ROOT={ref_root}"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return REF_LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        _lib = C.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


P = C.c_void_p
I = C.c_int
F = C.c_float
D = C.c_double
UL = C.c_ulong
SZ = C.c_size_t


def _declare(L):
    L.orc_nd.restype = I
    L.orc_nd.argtypes = [F, F, F]
    L.orc_osm_nd.restype = UL
    L.orc_osm_nd.argtypes = [F, F, F]
    L.orc_min_order_one.restype = I
    L.orc_min_order_one.argtypes = [I]
    L.orc_min_order.restype = I
    L.orc_min_order.argtypes = [P, I]
    L.orc_choose_M.restype = I
    L.orc_choose_M.argtypes = [I, I]
    L.orc_delaycount.restype = I
    L.orc_delaycount.argtypes = [I, I]
    L.orc_segmentation.restype = I
    L.orc_segmentation.argtypes = [F, F, F, I, I, P]
    L.orc_build_segments.restype = I
    L.orc_build_segments.argtypes = [P, I, I, P, P, P]
    L.orc_response.restype = None
    L.orc_response.argtypes = [F, F, F, I, P]
    L.orc_response_derivative.restype = None
    L.orc_response_derivative.argtypes = [F, F, F, I, P]
    L.orc_osm_min_order.restype = UL
    L.orc_osm_min_order.argtypes = [UL]
    L.orc_decode_u16.argtypes = [P, SZ, P]
    L.orc_decode_i8.argtypes = [P, SZ, P]
    L.orc_encode_u16.argtypes = [P, SZ, P]
    L.orc_intensity1.argtypes = [P, SZ, P]
    L.orc_intensity2.argtypes = [P, P, SZ, P]
    L.orc_fold.argtypes = [P, SZ, UL, D, D, D, P, P]
    L.orc_fold_bin.restype = UL
    L.orc_fold_bin.argtypes = [D, D, D, UL, SZ]
    L.orc_fold_finalize.argtypes = [P, P, UL, P]
    for pre in ("orc64_", "orc32_"):
        getattr(L, pre + "msosm_create").restype = P
        getattr(L, pre + "msosm_create").argtypes = [I, I, I, P, P, I, I]
        getattr(L, pre + "msosm_destroy").argtypes = [P]
        getattr(L, pre + "msosm_set_fold").argtypes = [P, UL, F, F]
        getattr(L, pre + "msosm_process").argtypes = [P, P, P]
        getattr(L, pre + "msosm_fold_read").argtypes = [P, P, P]
        getattr(L, pre + "fft").argtypes = [P, I, I, I]


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------
# planning
# --------------------------------------------------------------------------
def nd(bw: float, dm: float, f0: float) -> int:
    return lib().orc_nd(bw, dm, f0)


def osm_nd(bw: float, dm: float, f0: float) -> int:
    return lib().orc_osm_nd(bw, dm, f0)


def min_order(nds) -> int:
    a = np.ascontiguousarray(nds, dtype=np.int32)
    return lib().orc_min_order(_p(a), len(a))


def choose_M(M_min: int, fftpoint: int) -> int:
    return lib().orc_choose_M(M_min, fftpoint)


def delaycount(nd_: int, M: int) -> int:
    return lib().orc_delaycount(nd_, M)


def segmentation(bw, f0, dm, nd_, M) -> tuple[np.ndarray, int]:
    d = np.zeros(2 * M, dtype=np.int32)
    dc = lib().orc_segmentation(bw, f0, dm, nd_, M, _p(d))
    return d, dc


def build_segments(delay: np.ndarray, maxlen: int = 256):
    delay = np.ascontiguousarray(delay, dtype=np.int32)
    F_ = len(delay)
    st = np.zeros(F_, np.int32)
    ln = np.zeros(F_, np.int32)
    gr = np.zeros(F_, np.int32)
    n = lib().orc_build_segments(_p(delay), F_, maxlen, _p(st), _p(ln), _p(gr))
    return st[:n].copy(), ln[:n].copy(), gr[:n].copy()


def response(bw, f0, dm, M) -> np.ndarray:
    H = np.zeros(2 * M, dtype=np.complex128)
    lib().orc_response(bw, f0, dm, M, _p(H))
    return H


def response_derivative(bw, f0, dm, M) -> np.ndarray:
    """dH/dDM (FP64), for the gradient checks."""
    H = np.zeros(2 * M, dtype=np.complex128)
    lib().orc_response_derivative(bw, f0, dm, M, _p(H))
    return H


def osm_min_order(nd_: int) -> int:
    return lib().orc_osm_min_order(nd_)


class Plan:
    """The processor's planning state (Prepare_MSOSM after initialize_uint16)."""

    def __init__(self, bw, f0, dms, fftpoint=0, batch=1, with_response=True):
        self.bw = np.float32(bw)
        self.f0 = np.float32(f0)
        self.dms = np.asarray(dms, dtype=np.float32)
        self.nd = np.array([nd(self.bw, float(d), self.f0) for d in self.dms], dtype=np.int32)
        self.M_min = min_order(self.nd)
        self.M = choose_M(self.M_min, fftpoint)
        self.F = 2 * self.M
        self.batch = batch
        self.delays = np.zeros((len(self.dms), self.F), dtype=np.int32)
        self.dc = np.zeros(len(self.dms), dtype=np.int32)
        for i, d in enumerate(self.dms):
            self.delays[i], self.dc[i] = segmentation(self.bw, self.f0, float(d), int(self.nd[i]), self.M)
        self.delaycount = int(self.dc.max()) if len(self.dc) else 0
        fbs = self.delaycount + batch - 1  # msosm_gpu_batch.cpp:113-117
        if fbs % batch:
            fbs += batch - fbs % batch
        self.fbs = max(fbs, batch)
        self.H = None
        if with_response:
            self.H = np.stack([response(self.bw, self.f0, float(d), self.M) for d in self.dms])


# --------------------------------------------------------------------------
# streaming processor
# --------------------------------------------------------------------------
class Msosm:
    """Streaming MS-OSM (FP64 when fp64=True, else the FP32 port)."""

    def __init__(self, plan: Plan, batch: int, fp64: bool = True, nthreads: int = 0,
                 H: np.ndarray | None = None):
        L = lib()
        self.fp64 = fp64
        self.pre = "orc64_" if fp64 else "orc32_"
        self.M, self.F, self.B, self.D = plan.M, plan.F, batch, len(plan.dms)
        fbs = plan.delaycount + batch - 1
        if fbs % batch:
            fbs += batch - fbs % batch
        self.fbs = max(fbs, batch)
        self.cdt = np.complex128 if fp64 else np.complex64
        Hs = plan.H if H is None else H
        self._H = np.ascontiguousarray(Hs, dtype=self.cdt)
        self._delays = np.ascontiguousarray(plan.delays, dtype=np.int32)
        nt = nthreads or (os.cpu_count() or 1)
        self.nthreads = nt
        self.h = getattr(L, self.pre + "msosm_create")(self.M, batch, self.D, _p(self._delays),
                                                      _p(self._H), self.fbs, nt)
        self.K = 0

    def set_fold(self, K: int, period: float, fs: float):
        getattr(lib(), self.pre + "msosm_set_fold")(self.h, K, period, fs)
        self.K = K

    def process(self, x: np.ndarray, want_output: bool = True) -> np.ndarray | None:
        x = np.ascontiguousarray(x, dtype=self.cdt)
        assert x.size == self.B * self.M
        out = np.zeros((self.D, self.B, self.M), dtype=self.cdt) if want_output else None
        getattr(lib(), self.pre + "msosm_process")(self.h, _p(x), _p(out) if out is not None else None)
        return out

    def fold_read(self):
        s = np.zeros((self.D, self.K), np.float64)
        c = np.zeros((self.D, self.K), np.uint64)
        getattr(lib(), self.pre + "msosm_fold_read")(self.h, _p(s), _p(c))
        return s, c

    def close(self):
        if self.h:
            getattr(lib(), self.pre + "msosm_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------
# codecs, fold, fft
# --------------------------------------------------------------------------
def decode_u16(packed: np.ndarray) -> np.ndarray:
    packed = np.ascontiguousarray(packed, dtype=np.uint32)
    out = np.zeros(packed.size, np.complex64)
    lib().orc_decode_u16(_p(packed), packed.size, _p(out))
    return out


def decode_i8(iq: np.ndarray) -> np.ndarray:
    iq = np.ascontiguousarray(iq, dtype=np.int8)
    out = np.zeros(iq.size // 2, np.complex64)
    lib().orc_decode_i8(_p(iq), iq.size // 2, _p(out))
    return out


def encode_u16(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex64)
    out = np.zeros(x.size, np.uint32)
    lib().orc_encode_u16(_p(x), x.size, _p(out))
    return out


def intensity1(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex64)
    out = np.zeros(a.size, np.float32)
    lib().orc_intensity1(_p(a), a.size, _p(out))
    return out


def intensity2(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex64)
    b = np.ascontiguousarray(b, dtype=np.complex64)
    out = np.zeros(a.size, np.float32)
    lib().orc_intensity2(_p(a), _p(b), a.size, _p(out))
    return out


def fold(inten: np.ndarray, K: int, t_start: float, dt: float, period: float, sum_=None, cnt=None):
    inten = np.ascontiguousarray(inten, dtype=np.float32)
    s = np.zeros(K, np.float64) if sum_ is None else sum_
    c = np.zeros(K, np.uint64) if cnt is None else cnt
    lib().orc_fold(_p(inten), inten.size, K, t_start, dt, period, _p(s), _p(c))
    return s, c


def fold_bin(t_start, dt, period, K, i) -> int:
    return lib().orc_fold_bin(t_start, dt, period, K, i)


def fold_finalize(s: np.ndarray, c: np.ndarray) -> np.ndarray:
    s = np.ascontiguousarray(s, np.float64)
    c = np.ascontiguousarray(c, np.uint64)
    out = np.zeros(s.shape, np.float32)
    lib().orc_fold_finalize(_p(s), _p(c), s.size, _p(out))
    return out


def fft(x: np.ndarray, sign: int = -1, fp64: bool = True) -> np.ndarray:
    dt = np.complex128 if fp64 else np.complex64
    y = np.array(x, dtype=dt, copy=True, order="C")
    n = y.shape[-1]
    count = y.size // n
    getattr(lib(), ("orc64_" if fp64 else "orc32_") + "fft")(_p(y), n, sign, count)
    return y


# --------------------------------------------------------------------------
# the compiled reference planning sources (x86 build container only)
# --------------------------------------------------------------------------
_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        if not REF_LIB_PATH.exists():
            return None
        _ref = C.CDLL(str(REF_LIB_PATH))
        _ref.ref_msosm_order.argtypes = [F, F, P, I, I, P, P, P]
        _ref.ref_msosm_tables.argtypes = [F, F, P, I, I, P, P, P, P]
        _ref.ref_osm_plan.argtypes = [F, F, F, UL, P, P, P, P]
    return _ref


def ref_plan(bw, f0, dms, fftpoint=0, want_delays=True, want_H=True):
    R = ref_lib()
    dms = np.ascontiguousarray(dms, dtype=np.float32)
    n = len(dms)
    nd_ = np.zeros(n, np.int32)
    mmin = np.zeros(1, np.int32)
    m = np.zeros(1, np.int32)
    R.ref_msosm_order(bw, f0, _p(dms), n, fftpoint, _p(nd_), _p(mmin), _p(m))
    M = int(m[0])
    dc = np.zeros(n, np.int32)
    dcmax = np.zeros(1, np.int32)
    delays = np.zeros((n, 2 * M), np.int32) if want_delays else None
    H = np.zeros((n, 2 * M), np.complex64) if want_H else None
    R.ref_msosm_tables(bw, f0, _p(dms), n, M, _p(dc), _p(dcmax),
                       _p(delays) if want_delays else None, _p(H) if want_H else None)
    return dict(nd=nd_, M_min=int(mmin[0]), M=M, dc=dc, delaycount=int(dcmax[0]), delays=delays, H=H)


def ref_build_segments(delay: np.ndarray) -> np.ndarray:
    """The reference's MSOSM_GPU_BATCH::build_segments on one delay map: (n, 3) int32
    (start, len, group)."""
    L = C.CDLL(str(REF_SEG_LIB_PATH))
    L.ref_build_segments.argtypes = [P, I, P, I]
    d = np.ascontiguousarray(delay, dtype=np.int32)
    out = np.zeros((len(d), 3), np.int32)
    n = L.ref_build_segments(_p(d), len(d), _p(out), len(d))
    return out[:n].copy()


def ref_osm_plan(bw, dm, f0, fftpoint=0, want_H=True):
    R = ref_lib()
    nd_ = np.zeros(1, np.uint64)
    mmin = np.zeros(1, np.uint64)
    m = np.zeros(1, np.uint64)
    R.ref_osm_plan(bw, dm, f0, 0, _p(nd_), _p(mmin), _p(m), None)
    M = int(m[0])
    if fftpoint:
        M2 = max(fftpoint // 2, int(mmin[0]))
    else:
        M2 = M
    H = np.zeros(2 * M2, np.complex64) if want_H else None
    R.ref_osm_plan(bw, dm, f0, fftpoint, _p(nd_), _p(mmin), _p(m), _p(H) if want_H else None)
    return dict(nd=int(nd_[0]), M_min=int(mmin[0]), M=int(m[0]), H=H)
