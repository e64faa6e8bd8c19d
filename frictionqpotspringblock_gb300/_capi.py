"""ctypes binding of the C ABI declared in include/fqsb.h (libfqsb.so).

The library is built in-tree (frictionqpotspringblock_gb300/_build/libfqsb.so).
Importing this module fails loudly when the library is missing: there is no
CPU fallback for any entry point.
"""

from __future__ import annotations

import ctypes
import pathlib

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libfqsb.so"

OK = 0
ERR_NAN = 1
ERR_NO_CONVERGENCE = 2
ERR_INVALID = 3
ERR_CUDA = 4
ERR_TIMEOUT = 5
ERR_NOT_POSSIBLE = 6
ERR_REQUIRE = 7
ERR_UNSUPPORTED = 8
ERR_NO_DEVICE = 9

CUSPY, SEMISMOOTH, SMOOTH = 0, 1, 2
INTERACTIONS_NONE, LAPLACE1D, LAPLACE2D, QUARTIC1D, QUARTICGRADIENT1D, QUARTICGRADIENT2D, LONGRANGE1D = range(7)
DISTRIBUTIONS = {
    "random": 0,
    "delta": 1,
    "exponential": 2,
    "power": 3,
    "gamma": 4,
    "pareto": 5,
    "weibull": 6,
    "normal": 7,
}
FIELD_U, FIELD_V, FIELD_A, FIELD_F, FIELD_F_POTENTIAL, FIELD_F_INTERACTIONS, FIELD_F_FRAME, FIELD_F_DAMPING = range(8)
SCALAR_U_FRAME, SCALAR_T, SCALAR_TEMPERATURE, SCALAR_RESIDUAL, SCALAR_MEAN_F_FRAME = range(5)
NOALLOC_MAX_N = 1 << 25  # FQSB_NOALLOC_MAX_N of include/fqsb.h


class Config(ctypes.Structure):
    _fields_ = [
        ("potential", ctypes.c_int),
        ("interactions", ctypes.c_int),
        ("rows", ctypes.c_int64),
        ("cols", ctypes.c_int64),
        ("m", ctypes.c_double),
        ("eta", ctypes.c_double),
        ("mu", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("k_interactions", ctypes.c_double),
        ("k_frame", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("distribution", ctypes.c_int),
        ("n_parameters", ctypes.c_int),
        ("parameters", ctypes.c_double * 4),
        ("offset", ctypes.c_double),
        ("offset_per_particle", ctypes.POINTER(ctypes.c_double)),
        ("nchunk", ctypes.c_int64),
        ("stream", ctypes.c_void_p),
        ("device", ctypes.c_int),
        ("interaction_parameters", ctypes.c_double * 2),
    ]


class BatchConfig(ctypes.Structure):
    _fields_ = [
        ("n_instances", ctypes.c_int64),
        ("sizes", ctypes.POINTER(ctypes.c_int64)),
        ("seeds", ctypes.POINTER(ctypes.c_uint64)),
        ("k_frame", ctypes.POINTER(ctypes.c_double)),
        ("m", ctypes.c_double),
        ("eta", ctypes.c_double),
        ("mu", ctypes.c_double),
        ("k_interactions", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("distribution", ctypes.c_int),
        ("n_parameters", ctypes.c_int),
        ("parameters", ctypes.c_double * 4),
        ("offset", ctypes.c_double),
        ("nchunk", ctypes.c_int64),
        ("window", ctypes.c_int64),
        ("threads", ctypes.c_int),
        ("ppt", ctypes.c_int),
        ("stream", ctypes.c_void_p),
        ("device", ctypes.c_int),
    ]


# (name, restype, argtypes) of every entry point of include/fqsb.h
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_PD = ctypes.POINTER(ctypes.c_double)
_PI64 = ctypes.POINTER(ctypes.c_int64)
_PU64 = ctypes.POINTER(ctypes.c_uint64)

SIGNATURES = [
    ("fqsb_create", _I, [ctypes.POINTER(Config), ctypes.POINTER(_P)]),
    ("fqsb_destroy", _I, [_P]),
    ("fqsb_last_error", ctypes.c_char_p, [_P]),
    ("fqsb_size", _I, [_P, _PI64]),
    ("fqsb_time_step", _I, [_P]),
    ("fqsb_time_steps", _I, [_P, _U64]),
    ("fqsb_flow_steps", _I, [_P, _U64, _D]),
    ("fqsb_time_steps_until_event", _I, [_P, _D, _U64, _U64, _PU64]),
    ("fqsb_minimise", _I, [_P, _D, _U64, _U64, _I, _I, _PU64]),
    ("fqsb_minimise_truncate", _I, [_P, _PI64, _U64, _U64, _D, _U64, _U64, _I, _I, _PU64]),
    ("fqsb_minimise_nopassing", _I, [_P, _D, _U64, _U64, _I, _PU64]),
    ("fqsb_max_uniform_displacement", _I, [_P, _I, _PD]),
    ("fqsb_event_driven_step", _I, [_P, _D, _I, _I, _PD]),
    ("fqsb_trigger", _I, [_P, _I64, _D, _I]),
    ("fqsb_advance_to_fixed_force", _I, [_P, _D, _I]),
    ("fqsb_quench", _I, [_P]),
    ("fqsb_refresh", _I, [_P]),
    ("fqsb_get_field", _I, [_P, _I, _PD]),
    ("fqsb_set_field", _I, [_P, _I, _PD]),
    ("fqsb_get_scalar", _I, [_P, _I, _PD]),
    ("fqsb_set_u_frame", _I, [_P, _D]),
    ("fqsb_get_inc", _I, [_P, _PI64]),
    ("fqsb_set_inc", _I, [_P, _I64]),
    ("fqsb_set_t", _I, [_P, _D]),
    ("fqsb_quasistatic_activity", _I, [_P, _PI64, _PI64]),
    ("fqsb_get_index", _I, [_P, _PI64, _PI64, _PD, _PD]),
    ("fqsb_chunk_size", _I, [_P, _PI64]),
    ("fqsb_chunk_data", _I, [_P, _PD, _PI64]),
    ("fqsb_chunk_state_at", _I, [_P, _PI64, _PU64]),
    ("fqsb_chunk_restore", _I, [_P, _PU64, _PD, _PI64]),
    ("fqsb_get_field_device", _I, [_P, _I, _P]),
    ("fqsb_set_field_device", _I, [_P, _I, _P]),
    ("fqsb_get_stream", _I, [_P, ctypes.POINTER(_P)]),
    ("fqsb_residual_noalloc", _I, [_P, _P, _I64, _P, _P]),
    ("fqsb_set_parameters", _I, [_P, _D, _D, _D]),
    ("fqsb_set_random_forcing", _I, [_P, _D, _D, _U64, _PI64, _PI64]),
    ("fqsb_random_forcing_get", _I, [_P, _PU64, _PD, _PI64]),
    ("fqsb_random_forcing_set", _I, [_P, _PU64, _PD, _PI64]),
    ("fqsb_adjoint_forward", _I, [_P, _PD, _I64, _I64, _I64, _PD]),
    ("fqsb_adjoint_backward", _I, [_P, _PD, _PD, _PD, _PD]),
    ("fqsb_adjoint_backward_device", _I, [_P, _P, _P, _PD, _PD]),
    ("fqsb_batch_create", _I, [ctypes.POINTER(BatchConfig), ctypes.POINTER(_P)]),
    ("fqsb_batch_destroy", _I, [_P]),
    ("fqsb_batch_last_error", ctypes.c_char_p, [_P]),
    ("fqsb_batch_quasistatic", _I, [_P, _I64, _D, _D, _U64, _U64, _PD, _PD, _PI64, _PI64, ctypes.POINTER(ctypes.c_int32)]),
    ("fqsb_batch_get", _I, [_P, _I64, _I, _PD]),
    ("fqsb_batch_get_index", _I, [_P, _I64, _PI64]),
    ("fqsb_batch_frame", _I, [_P, _PD]),
    ("fqsb_measure_arith", _I, [_I, _I, _I, _PD]),
    ("fqsb_version", ctypes.c_char_p, []),
]

_lib = None


def lib() -> ctypes.CDLL:
    """Load libfqsb.so (built by __graft_entry__.build() or _build_lib.build())."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')"
            )
        L = ctypes.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def measure_arith(op: str = "add", n_soft: int = 0, device: int = 0) -> float:
    """Binary64 operations per second (Gop/s) of this GPU for op "add", "mul" or "fma", with n_soft of
    8 independent chains per thread in the integer-pipe form of the step kernels (fqsb_measure_arith)."""
    out = ctypes.c_double()
    check(None, lib().fqsb_measure_arith(int(device), {"add": 0, "mul": 1, "fma": 2}[op], int(n_soft),
                                         ctypes.byref(out)))
    return out.value


def exported_symbols() -> list[str]:
    return [s[0] for s in SIGNATURES]


class FrictionError(RuntimeError):
    """Raised for every non-zero status; the message reproduces the reference's exception text."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def check(handle, status: int):
    if status != OK:
        msg = lib().fqsb_last_error(handle)
        raise FrictionError(status, msg.decode() if msg else f"fqsb status {status}")
