"""ctypes binding of libbpl_gb300.so (the C ABI declared in include/bpl_gb300.h).

The library is built in-tree by bpl_gb300._build.build() (called by
__graft_entry__.build()).  There is no fallback: if the library is missing
every op raises.
"""
from __future__ import annotations

import ctypes
import os

from ._build import LIB_PATH

_lib = None

c_int, c_float, c_void_p = ctypes.c_int, ctypes.c_float, ctypes.c_void_p

# name -> argtypes (all functions return int status unless listed in _RESTYPE)
SIGNATURES = {
    "bpl_version": [],
    "bpl_status_string": [c_int],
    "bpl_last_error": [],
    "bpl_read_device_error": [c_void_p],
    "bpl_set_wait_limit": [ctypes.c_uint],
    "bpl_lbp_forward": [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p] + [c_int] * 8 + [c_void_p],
    "bpl_lbp_forward_f16": [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p] + [c_int] * 8 + [c_void_p],
    "bpl_lbp_backward_workspace_size": [c_int] * 4,
    "bpl_lbp_backward": [c_int] + [c_void_p] * 5 + [c_int] + [c_void_p] * 5 + [ctypes.c_size_t] + [c_int] * 7 + [c_void_p],
    "bpl_lbp_backward_f16": [c_int] + [c_void_p] * 5 + [c_int] + [c_void_p] * 5 + [ctypes.c_size_t] + [c_int] * 7 + [c_void_p],
    "bpl_lbp_backward_exact": [c_int] + [c_void_p] * 5 + [c_int] + [c_void_p] * 6 + [ctypes.c_size_t] + [c_int] * 7 + [c_void_p],
    "bpl_lbp_backward_passes": [c_int] + [c_void_p] * 3 + [ctypes.c_int64] * 2 + [c_void_p] * 2 + [c_int] + [c_void_p] * 5 + [ctypes.c_size_t] + [c_int] * 8 + [c_void_p],
    "bpl_lbp_backward_passes_f16": [c_int] + [c_void_p] * 3 + [ctypes.c_int64] * 2 + [c_void_p] * 2 + [c_int] + [c_void_p] * 5 + [ctypes.c_size_t] + [c_int] * 8 + [c_void_p],
    "bpl_beliefs_forward": [c_void_p, c_int] + [c_void_p] * 3 + [c_int] * 5 + [c_void_p],
    "bpl_beliefs_backward": [c_void_p, c_int] + [c_void_p] * 6 + [c_int] * 5 + [c_void_p],
    "bpl_lbp_backward_passes_into": [c_int, c_int] + [c_void_p] * 3 + [ctypes.c_int64] * 2 + [c_void_p] * 2 + [c_int] + [c_void_p] * 2 + [c_int, c_float] + [c_void_p] * 3 + [ctypes.c_size_t] + [c_int] * 9 + [c_void_p],
    "bpl_beliefs_forward_ex": [c_void_p, c_int, c_void_p, c_int, c_float] + [c_void_p] * 3 + [c_int] * 5 + [c_void_p],
    "bpl_beliefs_backward_ex": [c_void_p, c_int, c_void_p, c_int, c_float] + [c_void_p] * 4 + [c_float, c_void_p, c_int, c_void_p, c_void_p] + [c_int] * 5 + [c_void_p],
    "bpl_half_padded": [c_void_p, c_float, c_void_p, ctypes.c_int64, c_int, c_int, c_void_p],
    "bpl_sad_volume_depth": [c_int, c_int, c_float],
    "bpl_sad_forward": [c_void_p] * 3 + [c_int] * 6 + [c_float, c_void_p],
    "bpl_sad_backward": [c_void_p] * 5 + [c_int] * 7 + [c_void_p],
    "bpl_flow_forward": [c_void_p] * 6 + [c_int] * 9 + [c_void_p],
    "bpl_flow_backward": [c_void_p] * 8 + [c_int] * 5 + [c_void_p],
    "bpl_flow_backward_workspace_size": [c_int] * 4,
    "bpl_broadcast_slots": [c_void_p] * 2 + [c_int, ctypes.c_int64, c_int, c_void_p],
    "bpl_upsample_add_beliefs": [c_void_p] * 2 + [c_int] * 4 + [ctypes.c_float, c_void_p],
    "bpl_flow_backward_ws": [c_void_p] * 9 + [ctypes.c_size_t] + [c_int] * 5 + [c_void_p],
    "bpl_cost_from_sad": [c_void_p, c_void_p, c_int] + [c_int] * 5 + [c_float, c_void_p],
    "bpl_messages_argmin": [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int] + [c_int] * 6 + [c_void_p],
    "bpl_beliefs_infer": [c_void_p, c_int, c_int, c_void_p] + [c_int] * 4 + [c_void_p],
    "bpl_pack_taps": [c_void_p] * 3 + [c_int] * 4 + [c_void_p],
    "bpl_unpack_tap_grad": [c_void_p] * 3 + [c_int] * 4 + [c_void_p],
    "bpl_lbp_backward_noalloc": [c_int] + [c_void_p] * 5 + [c_int] + [c_void_p] * 4 + [c_int] * 7 + [c_void_p],
}
_RESTYPE = {"bpl_status_string": ctypes.c_char_p, "bpl_last_error": ctypes.c_char_p,
            "bpl_lbp_backward_workspace_size": ctypes.c_size_t,
            "bpl_flow_backward_workspace_size": ctypes.c_size_t}


class BplError(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise BplError(
                "libbpl_gb300.so is not built (expected at %s); run bpl_gb300._build.build() "
                "or __graft_entry__.build() first" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, c_int)
        _lib = L
    return _lib


def check(status: int, what: str) -> None:
    if status != 0:
        L = lib()
        raise BplError("%s failed: %s: %s" % (what, L.bpl_status_string(status).decode(),
                                                L.bpl_last_error().decode()))


def read_device_error() -> int:
    """Synchronises the current device, returns and clears the device error
    word (0: no kernel's bounded wait ran out since the last read)."""
    code = ctypes.c_int(0)
    check(lib().bpl_read_device_error(ctypes.byref(code)), "bpl_read_device_error")
    return code.value


DEVICE_ERRORS = {1: "a kernel's bounded wait for its staged input ran out (device wait timeout)"}


def check_device_error() -> None:
    """Raises BplError if a kernel launched since the last check reported a
    device error; the outputs of those launches are then incomplete.  The
    launches themselves do not synchronise, so callers check at a point
    where they synchronise anyway (a loss read back to the host, the end of
    an epoch or of a served batch).  Synchronises the current device."""
    code = read_device_error()
    if code:
        raise BplError("device error %d: %s" % (code, DEVICE_ERRORS.get(code, "unknown")))


DEFAULT_WAIT_LIMIT = 1 << 24


def set_wait_limit(polls: int | None) -> None:
    """Poll limit of the kernels' bounded waits on the current device (None:
    the default; 0: every wait gives up at once).  For tests of the timeout
    path."""
    check(lib().bpl_set_wait_limit(DEFAULT_WAIT_LIMIT if polls is None else int(polls)), "bpl_set_wait_limit")
