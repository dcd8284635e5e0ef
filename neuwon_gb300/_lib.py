"""ctypes binding of ``libneuwon_gb300.so`` (the C ABI in include/neuwon_gb300.h).

There is no fallback: if the library is missing or no CUDA device is present,
the calls raise.  ``load()`` builds the library on first use when the CUDA
toolkit is available.
"""
import ctypes
import os

import numpy as np

from .build import LIB, build

NW_OK = 0
NW_F32, NW_F64 = 4, 8
DTYPES = {np.dtype(np.float64): 1, np.dtype(np.float32): 2, np.dtype(np.int64): 3,
          np.dtype(np.int32): 4, np.dtype(np.uint32): 5, np.dtype(np.uint8): 6,
          np.dtype(np.bool_): 6}
PATH_BATCHED, PATH_PLAIN, PATH_WIDE = 0, 1, 2

EXPORTS = [
    "nw_version", "nw_ctx_create", "nw_ctx_destroy", "nw_last_error", "nw_get_stream",
    "nw_synchronize", "nw_model_init", "nw_set_data", "nw_get_data", "nw_propagator_build",
    "nw_propagator_set_csr", "nw_propagator_get_csr", "nw_hh_register", "nw_clamps_set",
    "nw_detectors_set", "nw_probes_set", "nw_probes_read", "nw_advance", "nw_advance_host", "nw_advance_host_async",
    "nw_get_clock", "nw_set_tuning", "nw_get_tuning", "nw_propagator_stats", "nw_propagator_conserve",
    "nw_kinetic_register", "nw_set_option", "nw_get_option", "nw_electric_half_step_noalloc",
    "nw_adjoint_forward", "nw_adjoint_backward", "nw_autotune", "nw_synapses_set",
    "nw_calcium_set", "nw_calcium_pump_set", "nw_calcium_data", "nw_lti_table_build", "nw_lti_expm",
    "nw_species_set", "nw_species_conductance", "nw_kinetic_add", "nw_kinetic_clear", "nw_kinetic_inputs",
]

_lib = None


class NeuwonError(RuntimeError):
    """A C-ABI call returned an error status."""


def load(build_if_missing=True):
    """Load (building first if needed) the shared library; raises if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        build()
    if not os.path.exists(LIB):
        raise ImportError(f"neuwon_gb300 CUDA library not found at {LIB}; run python -m neuwon_gb300.build")
    lib = ctypes.CDLL(LIB)
    c_void_p, c_int, c_i64, c_double = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    P = ctypes.POINTER
    sig = {
        "nw_version": ([], c_int),
        "nw_ctx_create": ([c_int, c_int, P(c_void_p)], c_int),
        "nw_ctx_destroy": ([c_void_p], c_int),
        "nw_last_error": ([c_void_p, ctypes.c_char_p, c_int], c_int),
        "nw_get_stream": ([c_void_p, P(c_void_p)], c_int),
        "nw_synchronize": ([c_void_p], c_int),
        "nw_model_init": ([c_void_p, c_i64, c_i64, c_void_p, c_void_p, c_double, c_double], c_int),
        "nw_set_data": ([c_void_p, ctypes.c_char_p, c_void_p, c_int, c_i64], c_int),
        "nw_get_data": ([c_void_p, ctypes.c_char_p, c_void_p, c_int, c_i64], c_int),
        "nw_propagator_build": ([c_void_p, c_double, P(c_i64)], c_int),
        "nw_propagator_set_csr": ([c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_i64], c_int),
        "nw_propagator_get_csr": ([c_void_p, c_void_p, c_void_p, c_void_p, P(c_i64)], c_int),
        "nw_propagator_conserve": ([c_void_p], c_int),
        "nw_hh_register": ([c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_void_p,
                            c_double, c_double, c_double, c_double], c_int),
        "nw_kinetic_register": ([c_void_p, c_i64, c_void_p, c_void_p, c_int, c_int, c_void_p, c_double,
                                 c_void_p, c_int, c_int, c_double, c_double, c_double, c_void_p], c_int),
        "nw_kinetic_add": ([c_void_p, c_i64, c_void_p, c_void_p, c_int, c_int, c_void_p, c_double, ctypes.c_int32,
                            c_void_p, c_int, c_int, c_double, c_double, c_double, c_void_p, P(ctypes.c_int32)], c_int),
        "nw_kinetic_clear": ([c_void_p], c_int),
        "nw_kinetic_inputs": ([c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, c_double, c_double, c_double,
                               ctypes.c_int32, ctypes.c_int32, c_double, c_double, c_double, ctypes.c_int32, c_void_p,
                               c_double], c_int),
        "nw_species_set": ([c_void_p, ctypes.c_int32, c_void_p], c_int),
        "nw_species_conductance": ([c_void_p, ctypes.c_int32, c_void_p], c_int),
        "nw_clamps_set": ([c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_void_p], c_int),
        "nw_detectors_set": ([c_void_p, c_void_p, c_void_p], c_int),
        "nw_probes_set": ([c_void_p, c_i64, c_void_p, c_i64], c_int),
        "nw_probes_read": ([c_void_p, c_void_p, c_int, c_i64, P(c_i64)], c_int),
        "nw_advance": ([c_void_p, ctypes.c_int32, c_int], c_int),
        "nw_advance_host": ([c_void_p, ctypes.c_int32, c_void_p, c_void_p, c_int], c_int),
        "nw_advance_host_async": ([c_void_p, ctypes.c_int32, c_void_p, c_void_p, c_int], c_int),
        "nw_get_clock": ([c_void_p, P(c_i64), P(c_i64)], c_int),
        "nw_set_tuning": ([c_void_p, c_int, c_int, c_int], c_int),
        "nw_set_option": ([c_void_p, ctypes.c_char_p, c_i64], c_int),
        "nw_get_option": ([c_void_p, ctypes.c_char_p, P(c_i64)], c_int),
        "nw_electric_half_step_noalloc": ([c_i64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                           c_void_p, c_void_p, c_void_p, c_void_p, c_double, c_void_p], c_int),
        "nw_adjoint_forward": ([c_void_p, c_i64, ctypes.c_int32, c_void_p, P(c_double)], c_int),
        "nw_adjoint_backward": ([c_void_p, c_double, c_void_p, c_void_p, c_void_p, P(c_double)], c_int),
        "nw_get_tuning": ([c_void_p, P(c_int), P(c_int), P(c_int)], c_int),
        "nw_synapses_set": ([c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_void_p, c_void_p, c_void_p, ctypes.c_int32, c_double, c_double], c_int),
        "nw_calcium_set": ([c_void_p, c_double, c_void_p, c_void_p, c_void_p, c_double, c_double, c_int,
                            P(c_i64)], c_int),
        "nw_calcium_pump_set": ([c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_int32, ctypes.c_int32,
                                 c_double, c_double, c_double, c_void_p], c_int),
        "nw_calcium_data": ([c_void_p, ctypes.c_char_p, c_void_p, c_int, c_i64, c_int], c_int),
        "nw_lti_table_build": ([c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, c_void_p,
                                c_void_p, c_double, ctypes.c_int32, c_void_p], c_int),
        "nw_lti_expm": ([c_void_p, ctypes.c_int32, c_i64, c_void_p, c_double, c_void_p], c_int),
        "nw_autotune": ([c_void_p, ctypes.c_int32, P(ctypes.c_int32), P(ctypes.c_int32), P(ctypes.c_int32),
                         P(c_double)], c_int),
        "nw_propagator_stats": ([c_void_p, P(c_i64), P(c_i64), P(c_i64), P(c_i64)], c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def ptr(a):
    """Data pointer of a C-contiguous numpy array (or None).  The returned ctypes
    object keeps a reference to the array, so a temporary passed inline stays
    alive for the duration of the call."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One device context of the library: owns the device mirror of a model."""

    def __init__(self, device=0, precision="f32"):
        self.lib = load()
        self.precision = {"f32": NW_F32, "f64": NW_F64}[precision]
        self.real = np.float32 if self.precision == NW_F32 else np.float64
        h = ctypes.c_void_p()
        rc = self.lib.nw_ctx_create(int(device), self.precision, ctypes.byref(h))
        if rc != NW_OK or not h.value:
            raise NeuwonError(f"nw_ctx_create(device={device}) failed with status {rc} "
                              "(is a CUDA device present?)")
        self.handle = h

    def check(self, rc, what):
        if rc != NW_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.nw_last_error(self.handle, buf, 512)
            raise NeuwonError(f"{what}: status {rc}: {buf.value.decode(errors='replace')}")

    def call(self, name, *args):
        self.check(getattr(self.lib, name)(self.handle, *args), name)

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.nw_ctx_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- typed helpers ---------------------------------------------------
    def set_data(self, name, values):
        a = np.ascontiguousarray(values)
        if a.dtype not in DTYPES:
            a = a.astype(np.float64)
        self.call("nw_set_data", name.encode(), ptr(a), DTYPES[a.dtype], a.size)

    def get_data(self, name, count, dtype=np.float64):
        out = np.empty(count, dtype=dtype)
        self.call("nw_get_data", name.encode(), ptr(out), DTYPES[out.dtype], count)
        return out

    def advance(self, k_steps=1, path=PATH_BATCHED):
        self.call("nw_advance", int(k_steps), int(path))

    def clock(self):
        s, t = ctypes.c_int64(), ctypes.c_int64()
        self.call("nw_get_clock", ctypes.byref(s), ctypes.byref(t))
        return s.value, t.value

    def set_option(self, name, value):
        self.call("nw_set_option", name.encode(), int(value))

    def get_option(self, name):
        v = ctypes.c_int64()
        self.call("nw_get_option", name.encode(), ctypes.byref(v))
        return v.value

    def autotune(self, trial_steps=10):
        """Times the batched path's launch shapes on this model and keeps the fastest;
        returns dict(lanes_per_row, threads, fusion_depth, ms_per_step, lanes_split,
        narrow_neurons): with the quad format, neurons whose mean quads per row are
        below lanes_split (narrow_neurons of them) take half the lanes per row."""
        l, t, f = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        ms = ctypes.c_double()
        self.call("nw_autotune", int(trial_steps), ctypes.byref(l), ctypes.byref(t), ctypes.byref(f),
                  ctypes.byref(ms))
        return {"lanes_per_row": l.value, "threads": t.value, "fusion_depth": f.value,
                "ms_per_step": ms.value, "lanes_split": self.get_option("lanes_split"),
                "narrow_neurons": self.get_option("narrow_neurons")}

    def propagator_csr(self):
        nnz = ctypes.c_int64()
        self.call("nw_propagator_get_csr", None, None, None, ctypes.byref(nnz))
        return nnz.value
