"""ctypes binding of libchimera_gb300.so (the C ABI in include/chimera_gb300.h).

The library is built in-tree by ``chimera_gb300.build``; loading fails loudly
when it is missing or was built for another machine -- there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import threading

from . import buildlib as _build

P, I, D, N = "p", "i", "d", "n"  # pointer, int64, double, int32

_HEADER = os.path.join(os.path.dirname(_build.HERE), "include", "chimera_gb300.h")


def _parse_header(path: str) -> dict[str, tuple[str, str]]:
    """name -> (return kind, argument kinds) for every declaration of the C
    header, so the ctypes signatures can never drift from it."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"(int64_t|int|double|const char \*)\s*(chm_\w+)\s*\(([^;]*?)\)\s*;", text):
        kinds = ""
        if args.strip() != "void":
            for a in args.split(","):
                a = " ".join(a.split())
                if "*" in a:
                    kinds += P
                elif a.startswith("int64_t"):
                    kinds += I
                elif a.startswith("double"):
                    kinds += D
                elif a.startswith("float"):
                    kinds += "f"
                elif a.startswith("int"):
                    kinds += N
                else:
                    raise ValueError(f"unparsed argument {a!r} of {name}")
        out[name] = ({"int": "n", "int64_t": "i", "double": "d"}.get(ret, "s"), kinds)
    return out


_SIG = _parse_header(_HEADER)

_KIND = {P: C.c_void_p, I: C.c_int64, D: C.c_double, N: C.c_int, "f": C.c_float}


class ChimeraError(RuntimeError):
    """A C-ABI call of libchimera_gb300 returned an error status."""


_lock = threading.Lock()
_lib = None


def load(build_if_missing: bool = True):
    """Load (building if needed) the CUDA library and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise ChimeraError(f"libchimera_gb300.so not built ({path})")
            _build.build()
        lib = C.CDLL(path)
        for name, (ret, kinds) in _SIG.items():
            fn = getattr(lib, name)
            fn.argtypes = [_KIND[k] for k in kinds]
            fn.restype = {"n": C.c_int, "i": C.c_int64, "d": C.c_double, "s": C.c_char_p}[ret]
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    """Every symbol include/chimera_gb300.h declares."""
    return list(_SIG)


_prof = None  # name -> list of (start, end) CUDA events while profiling


def profile_begin():
    """Record CUDA events around every C-ABI call on the current stream."""
    global _prof
    _prof = {}


def profile_end() -> dict:
    """Stop recording; returns name -> (calls, total device ms, dense-product
    FLOPs issued by those calls)."""
    global _prof
    import torch
    prof, _prof = _prof, None
    torch.cuda.synchronize()
    return {k: (len(v), sum(a.elapsed_time(b) for a, b, _ in v), sum(f for _, _, f in v))
            for k, v in (prof or {}).items()}


def call(name: str, *args):
    """Call a status-returning entry point; raise ChimeraError on failure."""
    lib = load()
    if _prof is not None:
        import torch
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        f0 = lib.chm_gemm_flops()
        a.record()
        rc = getattr(lib, name)(*args)
        b.record()
        _prof.setdefault(name, []).append((a, b, lib.chm_gemm_flops() - f0))
    else:
        rc = getattr(lib, name)(*args)
    if rc != 0:
        msg = lib.chm_last_error().decode(errors="replace")
        raise ChimeraError(f"{name} failed with status {rc}: {msg}")
    return rc


def query(name: str, *args) -> int:
    return int(getattr(load(), name)(*args))
