"""Python binding of the GB300 MS-OSM engine's C ABI (include/msosm_gb300.h).

A thin ctypes layer used by the test-suite and bench.py: it loads the in-tree
shared library (acceleratedms-osm_gb300/lib/libmsosm_gb300.so) and raises if
it is missing -- there is no CPU fallback.  Device buffers may be passed as
integers (raw device pointers) or as torch CUDA tensors; host buffers as numpy
arrays or pinned torch CPU tensors.

Class names follow the reference's processors:
  MsosmGpuBatch  ~ MSOSM_GPU_BATCH (dedispersion/include/msosm_gpu_batch.h:13-97)
  OsmGpuBatch    ~ OSM_GPU_BATCH   (dedispersion/include/osm_gpu_batch.h:7-38)
  FoldGpu        ~ Fold_GPU        (folding/include/fold_gpu.h:10-43)
  Simulator      ~ SimulatedComplexSignal + AWGN (simulated_pulsar/include/*.h)
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parents[1]
LIB_PATH = PKG / "lib" / "libmsosm_gb300.so"
HEADER = PKG.parent / "include" / "msosm_gb300.h"

OK = 0
IN_U16, IN_C64, IN_I8 = 0, 1, 2
OUT_NONE, OUT_C64, OUT_U16 = 0, 1, 2
PREC_FP32, PREC_BF16X3, PREC_FP16X3 = 0, 1, 2
IN_BYTES = {IN_U16: 4, IN_C64: 8, IN_I8: 2}

_lib = None


class MsosmError(RuntimeError):
    pass


def build(force: bool = False) -> Path:
    import importlib.util

    spec = importlib.util.spec_from_file_location("_msosm_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def declared_functions() -> list[str]:
    """Function names declared in include/msosm_gb300.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:msosm|osm)_[a-z0-9_]+)\s*\(", text)))


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise MsosmError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        L = C.CDLL(str(LIB_PATH))
        _declare(L)
        _lib = L
    return _lib


P, I, F, D, UL, LL = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_ulong, C.c_longlong
PI = C.POINTER(C.c_int)


def _declare(L):
    L.msosm_version.restype = C.c_char_p
    L.msosm_status_string.restype = C.c_char_p
    L.msosm_status_string.argtypes = [I]
    L.msosm_create.argtypes = [F, F, P, I, C.POINTER(P)]
    L.osm_create.argtypes = [F, F, F, C.POINTER(P)]
    L.msosm_init.argtypes = [P, I, I, I, I]
    L.msosm_set_precision.argtypes = [P, I]
    L.msosm_get_launch_info.argtypes = [P, PI, PI, PI, PI]
    L.msosm_get_precision.argtypes = [P]
    L.msosm_get_dims.argtypes = [P, PI, PI, PI, PI, PI, PI, PI]
    L.msosm_get_nd.argtypes = [P, P]
    L.msosm_get_delaycounts.argtypes = [P, P]
    L.msosm_get_delay_points.argtypes = [P, I, P]
    L.msosm_get_response.argtypes = [P, I, P]
    L.msosm_process.argtypes = [P, P, P]
    L.msosm_process_many.argtypes = [P, P, I, P]
    L.msosm_get_output.argtypes = [P, P, P]
    L.msosm_device_output.restype = P
    L.msosm_device_output.argtypes = [P]
    L.msosm_device_output_u16.restype = P
    L.msosm_device_output_u16.argtypes = [P]
    L.msosm_steps.restype = LL
    L.msosm_steps.argtypes = [P]
    L.msosm_sync.argtypes = [P, P]
    L.msosm_destroy.argtypes = [P]
    L.msosm_last_error.restype = C.c_char_p
    L.msosm_last_error.argtypes = [P]
    L.msosm_fold_create.argtypes = [F, F, UL, UL, I, C.POINTER(P)]
    L.msosm_fold_accumulate.argtypes = [P, P, P, P]
    L.msosm_fold_read.argtypes = [P, P, P, P, P]
    L.msosm_fold_reset.argtypes = [P, P]
    L.msosm_fold_dims.argtypes = [P, C.POINTER(UL), PI, C.POINTER(UL)]
    L.msosm_fold_destroy.argtypes = [P]
    L.msosm_attach_fold.argtypes = [P, P]
    L.msosm_attach_fold_pol2.argtypes = [P, P, P]
    L.msosm_profile_enable.argtypes = [P, I]
    L.msosm_profile_reset.argtypes = [P]
    L.msosm_profile_read.argtypes = [P, I, C.POINTER(D), C.POINTER(LL), C.POINTER(LL), C.POINTER(LL)]
    L.msosm_state_bytes.restype = C.c_size_t
    L.msosm_state_bytes.argtypes = [P]
    L.msosm_save_state.argtypes = [P, P, C.c_size_t, P]
    L.msosm_load_state.argtypes = [P, P, C.c_size_t, P]
    L.msosm_fold_state_bytes.restype = C.c_size_t
    L.msosm_fold_state_bytes.argtypes = [P]
    L.msosm_fold_save_state.argtypes = [P, P, C.c_size_t, P]
    L.msosm_fold_load_state.argtypes = [P, P, C.c_size_t, P]
    L.msosm_plan_response_derivative.argtypes = [F, F, F, I, P]
    L.msosm_use_response_derivative.argtypes = [P]
    L.msosm_fold_accumulate_cross.argtypes = [P, P, P, P]
    L.msosm_writer_create.argtypes = [C.c_char_p, C.c_char_p, P, I, C.c_ulonglong, I, I, C.POINTER(P)]
    L.msosm_attach_writer.argtypes = [P, P]
    L.msosm_writer_write.argtypes = [P, P]
    L.msosm_writer_join.argtypes = [P]
    L.msosm_writer_last_error.restype = C.c_char_p
    L.msosm_writer_last_error.argtypes = [P]
    L.msosm_writer_filename.argtypes = [P, I, C.c_char_p, C.c_size_t]
    L.msosm_writer_destroy.argtypes = [P]
    L.msosm_plan_nd.argtypes = [F, F, P, I, P]
    L.msosm_plan_min_order.argtypes = [P, I, P]
    L.msosm_plan_segmentation.argtypes = [F, F, F, I, I, P, P]
    L.msosm_plan_response.argtypes = [F, F, F, I, P]
    L.osm_plan.argtypes = [F, F, F, C.POINTER(UL), C.POINTER(UL)]
    L.msosm_set_response.argtypes = [P, I, P]
    L.msosm_set_launch_shape.argtypes = [P, I, I]
    L.msosm_reset_l2_persisting.argtypes = []
    L.msosm_graph_create.argtypes = [P, P, I, C.POINTER(P)]
    L.msosm_graph_launch.argtypes = [P, P]
    L.msosm_graph_destroy.argtypes = [P]
    L.msosm_writer_copy_output.argtypes = [P, P, P]
    ULL = C.c_ulonglong
    L.msosm_sim_create.argtypes = [F, F, F, F, C.POINTER(P)]
    L.msosm_sim_set_pulse.argtypes = [P, I, F]
    L.msosm_sim_set_noise.argtypes = [P, I, F]
    L.msosm_sim_set_seed.argtypes = [P, ULL]
    L.msosm_sim_info.argtypes = [P, C.POINTER(ULL), C.POINTER(ULL), C.POINTER(D), C.POINTER(D)]
    L.msosm_sim_generate.argtypes = [P, ULL, I, F, P, P]
    L.msosm_sim_position.restype = ULL
    L.msosm_sim_position.argtypes = [P]
    L.msosm_sim_last_error.restype = C.c_char_p
    L.msosm_sim_last_error.argtypes = [P]
    L.msosm_sim_destroy.argtypes = [P]
    L.msosm_awgn.argtypes = [ULL, ULL, ULL, F, F, P, P]


def plan_nd(bw, f0, dms) -> np.ndarray:
    d = np.ascontiguousarray(np.atleast_1d(np.asarray(dms, np.float32)))
    out = np.zeros(len(d), np.int32)
    if lib().msosm_plan_nd(bw, f0, d.ctypes.data, len(d), out.ctypes.data) != OK:
        raise MsosmError("msosm_plan_nd")
    return out


def plan_min_order(nd) -> int:
    a = np.ascontiguousarray(np.atleast_1d(np.asarray(nd, np.int32)))
    m = np.zeros(1, np.int32)
    if lib().msosm_plan_min_order(a.ctypes.data, len(a), m.ctypes.data) != OK:
        raise MsosmError("msosm_plan_min_order")
    return int(m[0])


def plan_segmentation(bw, f0, dm, nd, M):
    d = np.zeros(2 * M, np.int32)
    dc = np.zeros(1, np.int32)
    if lib().msosm_plan_segmentation(bw, f0, dm, nd, M, d.ctypes.data, dc.ctypes.data) != OK:
        raise MsosmError("msosm_plan_segmentation")
    return d, int(dc[0])


def plan_response(bw, f0, dm, M) -> np.ndarray:
    H = np.zeros(2 * M, np.complex64)
    if lib().msosm_plan_response(bw, f0, dm, M, H.ctypes.data) != OK:
        raise MsosmError("msosm_plan_response")
    return H


def plan_response_derivative(bw, f0, dm, M) -> np.ndarray:
    H = np.zeros(2 * M, np.complex64)
    if lib().msosm_plan_response_derivative(bw, f0, dm, M, H.ctypes.data) != OK:
        raise MsosmError("msosm_plan_response_derivative")
    return H


def osm_plan(bw, dm, f0):
    nd, mm = C.c_ulong(), C.c_ulong()
    lib().osm_plan(bw, dm, f0, C.byref(nd), C.byref(mm))
    return nd.value, mm.value


def _ptr(x):
    """Raw address of a numpy array, torch tensor, int or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError(f"cannot take the address of {type(x)}")


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


class MsosmGpuBatch:
    """MS-OSM processor over many DM trials (MSOSM_GPU_BATCH)."""

    def __init__(self, bw: float, dms, f0: float, *, _osm_dm: float | None = None):
        L = lib()
        self._h = P()
        if _osm_dm is None:
            d = np.ascontiguousarray(np.atleast_1d(np.asarray(dms, dtype=np.float32)))
            rc = L.msosm_create(bw, f0, d.ctypes.data, len(d), C.byref(self._h))
            self.dms = d
        else:
            rc = L.osm_create(bw, _osm_dm, f0, C.byref(self._h))
            self.dms = np.array([_osm_dm], np.float32)
        if rc != OK:
            raise MsosmError(f"create failed: {L.msosm_status_string(rc).decode()}")
        self.num_dms = len(self.dms)
        self.nd = np.zeros(self.num_dms, np.int32)
        L.msosm_get_nd(self._h, self.nd.ctypes.data)
        self._fold = None
        self.inited = False

    # -- reference-shaped API ------------------------------------------------
    def initialize(self, fftpoint: int = 0, batch: int = 1, in_format: int = IN_U16, out_mode: int = OUT_C64):
        self._check(lib().msosm_init(self._h, fftpoint, batch, in_format, out_mode))
        self.in_format, self.out_mode = in_format, out_mode
        vals = [C.c_int() for _ in range(7)]
        lib().msosm_get_dims(self._h, *[C.byref(v) for v in vals])
        (self.M, self.M_min, self.fftpoint, self.batch, self.num_dms, self.delaycount,
         self.ring_blocks) = [v.value for v in vals]
        self.inited = True
        return self

    def filter_block(self, data, stream=None):
        """One step: batch*M samples (host array/pinned tensor or device tensor)."""
        self._check(lib().msosm_process(self._h, _ptr(data), _stream(stream)))

    def filter_blocks(self, data, nsteps: int, stream=None):
        self._check(lib().msosm_process_many(self._h, _ptr(data), nsteps, _stream(stream)))

    def get_output(self, out, stream=None):
        self._check(lib().msosm_get_output(self._h, _ptr(out), _stream(stream)))

    def get_output_pointer(self) -> int:
        return lib().msosm_device_output(self._h) or 0

    def get_output_pointer_u16(self) -> int:
        return lib().msosm_device_output_u16(self._h) or 0

    def synchronize(self, stream=None):
        self._check(lib().msosm_sync(self._h, _stream(stream)))

    def attach_fold(self, fold: "FoldGpu | None"):
        self._check(lib().msosm_attach_fold(self._h, fold._h if fold is not None else None))
        self._fold = fold

    def attach_fold_pol2(self, second: "MsosmGpuBatch", fold: "FoldGpu | None"):
        """2-pol fused fold: this handle is the first polarisation, `second` the other;
        each step process this one, then `second` (msosm_attach_fold_pol2)."""
        second._check(lib().msosm_attach_fold_pol2(self._h, second._h, fold._h if fold is not None else None))
        self._fold = fold
        second._fold = fold

    # -- checkpoint / derivative -------------------------------------------
    def save_state(self, stream=None) -> np.ndarray:
        n = lib().msosm_state_bytes(self._h)
        buf = np.zeros(n, np.uint8)
        self._check(lib().msosm_save_state(self._h, buf.ctypes.data, n, _stream(stream)))
        return buf

    def load_state(self, buf: np.ndarray, stream=None):
        self._check(lib().msosm_load_state(self._h, buf.ctypes.data, buf.nbytes, _stream(stream)))

    def set_precision(self, precision: int):
        """PREC_FP32 (default), PREC_BF16X3 or PREC_FP16X3: the inverse transforms' DFT
        stages on the tensor cores with split 16-bit operands (msosm_set_precision)."""
        self._check(lib().msosm_set_precision(self._h, int(precision)))
        return self

    def capture(self, data, nsteps: int) -> "StepGraph":
        """A CUDA graph of the next `nsteps` steps reading device buffer `data`
        (msosm_graph_create); launch() replays them as the following steps."""
        g = P()
        self._check(lib().msosm_graph_create(self._h, _ptr(data), int(nsteps), C.byref(g)))
        return StepGraph(self, g, data)

    def set_launch_shape(self, ctas_per_sm: int = 0, dm_group: int = 0) -> "MsosmGpuBatch":
        """Persistent transform: at most ctas_per_sm resident CTAs per SM (0 = all that fit)
        and DM trials in window-major groups of dm_group (0 = keep)."""
        self._check(lib().msosm_set_launch_shape(self._h, int(ctas_per_sm), int(dm_group)))
        return self

    def launch_info(self) -> dict:
        """Geometry of the last persistent inverse-transform launch."""
        v = [C.c_int() for _ in range(4)]
        self._check(lib().msosm_get_launch_info(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("grid", "occupancy", "lag", "slots"), (x.value for x in v)))

    @property
    def precision(self) -> int:
        return int(lib().msosm_get_precision(self._h))

    def use_response_derivative(self):
        """Outputs become dx/dDM (responses replaced by dH/dDM, delays unchanged)."""
        self._check(lib().msosm_use_response_derivative(self._h))

    # -- kernel timing ------------------------------------------------------
    KERNELS = ("fwd_pass1", "fwd_pass2", "inv_pass1", "inv_pass2", "inv_persistent")

    def profile(self, on: bool = True):
        self._check(lib().msosm_profile_enable(self._h, 1 if on else 0))

    def profile_reset(self):
        self._check(lib().msosm_profile_reset(self._h))

    def profile_read(self) -> dict:
        """{kernel: dict(ms, launches, timed, transforms)}; sync the stream first."""
        out = {}
        for k, name in enumerate(self.KERNELS):
            ms, n, t, tr = D(), LL(), LL(), LL()
            self._check(lib().msosm_profile_read(self._h, k, C.byref(ms), C.byref(n), C.byref(t), C.byref(tr)))
            out[name] = dict(ms=ms.value, launches=n.value, timed=t.value, transforms=tr.value)
        return out

    # -- planning results --------------------------------------------------
    @property
    def steps(self) -> int:
        return lib().msosm_steps(self._h)

    def delaycounts(self) -> np.ndarray:
        out = np.zeros(self.num_dms, np.int32)
        self._check(lib().msosm_get_delaycounts(self._h, out.ctypes.data))
        return out

    def delay_points(self, i: int) -> np.ndarray:
        out = np.zeros(self.fftpoint, np.int32)
        self._check(lib().msosm_get_delay_points(self._h, i, out.ctypes.data))
        return out

    def response(self, i: int) -> np.ndarray:
        out = np.zeros(self.fftpoint, np.complex64)
        self._check(lib().msosm_get_response(self._h, i, out.ctypes.data))
        return out

    def samples_per_step(self) -> int:
        return self.batch * self.M

    def _check(self, rc):
        if rc != OK:
            msg = lib().msosm_last_error(self._h)
            raise MsosmError(f"{lib().msosm_status_string(rc).decode()}: {msg.decode() if msg else ''}")

    def close(self):
        if self._h:
            lib().msosm_destroy(self._h)
            self._h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OsmGpuBatch(MsosmGpuBatch):
    """Plain overlap-save, single DM (OSM_GPU_BATCH)."""

    def __init__(self, bw: float, dm: float, f0: float):
        super().__init__(bw, None, f0, _osm_dm=dm)


class StepGraph:
    """Captured steps of a processor (msosm_graph_*); keeps the processor and the input alive."""

    def __init__(self, proc: MsosmGpuBatch, g, data):
        self.proc, self._g, self._data = proc, g, data

    def launch(self, stream=None):
        self.proc._check(lib().msosm_graph_launch(self._g, _stream(stream)))

    def __del__(self):
        if getattr(self, "_g", None) and _lib is not None:
            _lib.msosm_graph_destroy(self._g)
            self._g = None


SIM_TEST_PULSE, SIM_GAUSSIAN, SIM_IMPULSES = 0, 1, 2


class Simulator:
    """Dispersed-pulsar baseband generated on the GPU (msosm_sim_*): the
    simulated_pulsar front end with a counter-based seeded generator."""

    def __init__(self, bw: float, f0: float, dm: float, period: float, *, kind: int = SIM_TEST_PULSE,
                 duty: float = 0.05, snr_db: float | None = None, seed: int = 1):
        L = lib()
        self._h = P()
        rc = L.msosm_sim_create(bw, f0, dm, period, C.byref(self._h))
        if rc != OK:
            raise MsosmError(f"msosm_sim_create: {L.msosm_status_string(rc).decode()}")
        self._check(L.msosm_sim_set_pulse(self._h, kind, duty))
        self._check(L.msosm_sim_set_noise(self._h, int(snr_db is not None), float(snr_db or 0.0)))
        self._check(L.msosm_sim_set_seed(self._h, int(seed)))
        np_, nd = C.c_ulonglong(), C.c_ulonglong()
        ps, ns = C.c_double(), C.c_double()
        self._check(L.msosm_sim_info(self._h, C.byref(np_), C.byref(nd), C.byref(ps), C.byref(ns)))
        self.period_samples, self.nd = np_.value, nd.value
        self.signal_power, self.noise_sigma = ps.value, ns.value

    def _check(self, rc):
        if rc != OK:
            raise MsosmError(f"{lib().msosm_status_string(rc).decode()}: {lib().msosm_sim_last_error(self._h).decode()}")

    def generate(self, n: int, fmt: int = IN_C64, scale: float = 1.0, out=None, stream=None):
        """The next n samples, into `out` (host array or device tensor) or a new numpy array."""
        if out is None:
            dt = {IN_C64: np.complex64, IN_U16: np.uint32, IN_I8: np.int8}[fmt]
            out = np.zeros(n * (2 if fmt == IN_I8 else 1), dt)
        self._check(lib().msosm_sim_generate(self._h, int(n), fmt, float(scale), _ptr(out), _stream(stream)))
        return out

    @property
    def position(self) -> int:
        return int(lib().msosm_sim_position(self._h))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.msosm_sim_destroy(self._h)
            self._h = None


def reset_l2_persisting() -> None:
    """Return L2 lines marked persisting by the persistent transform to normal."""
    if lib().msosm_reset_l2_persisting() != OK:
        raise MsosmError("msosm_reset_l2_persisting")


def awgn(n: int, mean: float = 0.0, stddev: float = 1.0, seed: int = 1, first: int = 0, out=None, stream=None):
    """n complex samples with independent N(mean, stddev^2) quadratures (msosm_awgn)."""
    if out is None:
        out = np.zeros(n, np.complex64)
    if lib().msosm_awgn(int(seed), int(first), int(n), float(mean), float(stddev), _ptr(out), _stream(stream)) != OK:
        raise MsosmError("msosm_awgn")
    return out


class FoldGpu:
    """Intensity + phase fold (Fold_GPU), for num_series independent series."""

    def __init__(self, period: float, fs: float, size: int, time_bin: int = 0, num_series: int = 1):
        L = lib()
        self._h = P()
        rc = L.msosm_fold_create(period, fs, size, time_bin, num_series, C.byref(self._h))
        if rc != OK:
            raise MsosmError(f"fold create failed: {L.msosm_status_string(rc).decode()}")
        K = C.c_ulong()
        S = C.c_int()
        Z = C.c_ulong()
        L.msosm_fold_dims(self._h, C.byref(K), C.byref(S), C.byref(Z))
        self.time_bin, self.num_series, self.size = K.value, S.value, Z.value

    def accumulate(self, pol1, pol2=None, stream=None):
        rc = lib().msosm_fold_accumulate(self._h, _ptr(pol1), _ptr(pol2), _stream(stream))
        if rc != OK:
            raise MsosmError(f"fold accumulate: {lib().msosm_status_string(rc).decode()}")

    def read(self, stream=None):
        shape = (self.num_series, self.time_bin)
        folded = np.zeros(shape, np.float32)
        sums = np.zeros(shape, np.float64)
        cnts = np.zeros(shape, np.uint64)
        rc = lib().msosm_fold_read(self._h, folded.ctypes.data, sums.ctypes.data, cnts.ctypes.data,
                                   _stream(stream))
        if rc != OK:
            raise MsosmError(f"fold read: {lib().msosm_status_string(rc).decode()}")
        return folded, sums, cnts

    def accumulate_cross(self, x, dx, stream=None):
        """Fold 2 Re(conj(x) dx) (counted where |x|^2 != 0)."""
        rc = lib().msosm_fold_accumulate_cross(self._h, _ptr(x), _ptr(dx), _stream(stream))
        if rc != OK:
            raise MsosmError(f"fold accumulate_cross: {lib().msosm_status_string(rc).decode()}")

    def save_state(self, stream=None) -> np.ndarray:
        n = lib().msosm_fold_state_bytes(self._h)
        buf = np.zeros(n, np.uint8)
        if lib().msosm_fold_save_state(self._h, buf.ctypes.data, n, _stream(stream)) != OK:
            raise MsosmError("fold save_state")
        return buf

    def load_state(self, buf: np.ndarray, stream=None):
        if lib().msosm_fold_load_state(self._h, buf.ctypes.data, buf.nbytes, _stream(stream)) != OK:
            raise MsosmError("fold load_state")

    def read_folded(self, out: np.ndarray, stream=None):
        """Folded means only, into a caller-owned float32 [num_series][time_bin] array."""
        assert out.dtype == np.float32 and out.size == self.num_series * self.time_bin
        rc = lib().msosm_fold_read(self._h, out.ctypes.data, None, None, _stream(stream))
        if rc != OK:
            raise MsosmError(f"fold read: {lib().msosm_status_string(rc).decode()}")
        return out

    def reset(self, stream=None):
        lib().msosm_fold_reset(self._h, _stream(stream))

    def close(self):
        if self._h:
            lib().msosm_fold_destroy(self._h)
            self._h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Writer:
    """Per-DM output files (MSOSM_DataSave_Uring without liburing)."""

    def __init__(self, directory: str, prefix: str, dms, bytes_per_dm: int, slots: int = 4, direct_io: bool = False):
        L = lib()
        d = np.ascontiguousarray(np.atleast_1d(np.asarray(dms, np.float32)))
        self._h = P()
        rc = L.msosm_writer_create(str(directory).encode(), prefix.encode(), d.ctypes.data, len(d), bytes_per_dm,
                                   slots, 1 if direct_io else 0, C.byref(self._h))
        if rc != OK:
            raise MsosmError(f"writer create: {L.msosm_status_string(rc).decode()}")
        self.num_dms, self.bytes_per_dm = len(d), bytes_per_dm

    def filenames(self) -> list[str]:
        out = []
        for i in range(self.num_dms):
            buf = C.create_string_buffer(4096)
            lib().msosm_writer_filename(self._h, i, buf, 4096)
            out.append(buf.value.decode())
        return out

    def write(self, block: np.ndarray):
        assert block.nbytes == self.num_dms * self.bytes_per_dm
        if lib().msosm_writer_write(self._h, np.ascontiguousarray(block).ctypes.data) != OK:
            raise MsosmError("writer write")

    def join(self):
        rc = lib().msosm_writer_join(self._h)
        if rc != OK:
            raise MsosmError(f"writer: {lib().msosm_writer_last_error(self._h).decode()}")

    def attach_to(self, m: MsosmGpuBatch):
        m._check(lib().msosm_attach_writer(m._h, self._h))
        m._writer = self

    def close(self):
        if self._h:
            lib().msosm_writer_destroy(self._h)
            self._h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_dat(path) -> np.ndarray:
    """A per-DM .dat file as complex64: uint32 words, low 16 bits real, high 16
    imaginary, value - 32768 unless the code is 0 (python_check/check.py:5-53)."""
    w = np.fromfile(path, dtype=np.uint32)
    re = (w & 0xFFFF).astype(np.int64)
    im = (w >> 16).astype(np.int64)
    re = np.where(re != 0, re - 32768, 0)
    im = np.where(im != 0, im - 32768, 0)
    return (re + 1j * im).astype(np.complex64)


def autotune(bw, f0, dms, batch, in_format=IN_C64, min_fftpoint=1 << 16, max_fftpoint=1 << 20, steps=3,
             cache: str | Path | None = None) -> tuple[int, float]:
    """Fastest fftpoint for this DM list on this GPU (msosm_autotune), remembered in
    an optional JSON cache keyed by GPU, band, DM list, batch and input format."""
    import hashlib
    import json

    d = np.ascontiguousarray(np.sort(np.atleast_1d(np.asarray(dms, np.float32))))
    key = None
    if cache is not None:
        try:
            import torch

            gpu = torch.cuda.get_device_name(0)
        except Exception:
            gpu = "unknown"
        key = "|".join([gpu, f"{float(np.float32(bw))}", f"{float(np.float32(f0))}",
                        hashlib.sha1(d.tobytes()).hexdigest()[:16], str(batch), str(in_format),
                        str(min_fftpoint), str(max_fftpoint)])
        p = Path(cache)
        table = json.loads(p.read_text()) if p.exists() else {}
        if key in table:
            return int(table[key]["fftpoint"]), float(table[key]["rate"])
    best = C.c_int()
    rate = C.c_double()
    L = lib()
    L.msosm_autotune.argtypes = [F, F, P, I, I, I, I, I, I, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    rc = L.msosm_autotune(bw, f0, d.ctypes.data, len(d), batch, in_format, min_fftpoint, max_fftpoint, steps,
                          C.byref(best), C.byref(rate))
    if rc != OK:
        raise MsosmError(f"autotune: {L.msosm_status_string(rc).decode()}")
    if cache is not None:
        p = Path(cache)
        table = json.loads(p.read_text()) if p.exists() else {}
        table[key] = {"fftpoint": best.value, "rate": rate.value}
        p.write_text(json.dumps(table, indent=1))
    return best.value, rate.value


def autotune_shape(bw, f0, dms, batches=(2, 4, 8, 16, 32), in_format=IN_C64, min_fftpoint=1 << 16,
                   max_fftpoint=1 << 20, steps=3) -> dict:
    """Fastest (fftpoint, batch, CTAs per SM) for this DM list on this GPU
    (msosm_autotune_shape)."""
    d = np.ascontiguousarray(np.sort(np.atleast_1d(np.asarray(dms, np.float32))))
    bs = np.ascontiguousarray(np.asarray(batches, np.int32))
    out = [C.c_int() for _ in range(3)]
    rate = C.c_double()
    L = lib()
    L.msosm_autotune_shape.argtypes = [F, F, P, I, I, I, I, P, I, I, PI, PI, PI, C.POINTER(C.c_double)]
    rc = L.msosm_autotune_shape(bw, f0, d.ctypes.data, len(d), in_format, min_fftpoint, max_fftpoint, bs.ctypes.data,
                                len(bs), steps, *[C.byref(v) for v in out], C.byref(rate))
    if rc != OK:
        raise MsosmError(f"autotune_shape: {L.msosm_status_string(rc).decode()}")
    return {"fftpoint": out[0].value, "batch": out[1].value, "ctas_per_sm": out[2].value, "rate": rate.value}


def selftest_wait(preset: int, target: int, timeout_ns: int) -> tuple[bool, int]:
    """Run the persistent transform's bounded device-side wait alone on a counter preset
    to `preset` (nothing else writes it), waiting for `target` (msosm_selftest_wait).
    Returns (timed_out, elapsed_ns)."""
    L = lib()
    L.msosm_selftest_wait.argtypes = [C.c_uint, C.c_uint, C.c_ulonglong, C.POINTER(C.c_int),
                                      C.POINTER(C.c_ulonglong)]
    t = C.c_int()
    e = C.c_ulonglong()
    rc = L.msosm_selftest_wait(preset, target, timeout_ns, C.byref(t), C.byref(e))
    if rc != OK:
        raise MsosmError(f"selftest_wait: {L.msosm_status_string(rc).decode()}")
    return bool(t.value), int(e.value)


def selftest_umma(A: np.ndarray, B: np.ndarray, n: int = 64, b_row0: int = 0, bf16: bool = True) -> np.ndarray:
    """Tensor-core operand-layout self-test (msosm_selftest_umma): D = A x B[b_row0:b_row0+n]^T
    computed by tcgen05 MMAs from 16-bit operands (uint16 bit patterns, A 128 x 64, B 64 x 64)
    with FP32 accumulation.  Returns D (128 x n float32)."""
    L = lib()
    L.msosm_selftest_umma.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_int)]
    a = np.ascontiguousarray(A, dtype=np.uint16)
    b = np.ascontiguousarray(B, dtype=np.uint16)
    if a.shape != (128, 64) or b.shape != (64, 64):
        raise ValueError("A must be 128 x 64 and B 64 x 64")
    d = np.zeros((128, n), np.float32)
    t = C.c_int()
    rc = L.msosm_selftest_umma(int(bf16), n, b_row0, a.ctypes.data, b.ctypes.data, d.ctypes.data, C.byref(t))
    if rc != OK:
        raise MsosmError(f"selftest_umma: {L.msosm_status_string(rc).decode()}")
    if t.value:
        raise MsosmError("selftest_umma: the MMA wait timed out")
    return d
