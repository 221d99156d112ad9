"""The C ABI library loads, exports every function include/rtmc.h declares, and its
structs match the ctypes mirrors.  No GPU needed (no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from radiativetransfermontecarlo_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "rtmc.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(rtmc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = C.CDLL(str(_lib.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"


def test_struct_layout_matches_binding():
    lib = _lib.load()
    sizes = (C.c_int64 * 4)()
    assert lib.rtmc_abi_sizes(sizes) == 0
    assert list(sizes) == [C.sizeof(_lib.RtmcMaterial), C.sizeof(_lib.RtmcTablesInfo),
                           C.sizeof(_lib.RtmcProblem), C.sizeof(_lib.RtmcStats)]
    assert lib.rtmc_abi_version() == 2


def test_host_functions_report_errors():
    lib = _lib.load()
    h = C.c_void_p()
    m = _lib.RtmcMaterial()
    m.d = 4  # invalid dimension
    assert lib.rtmc_tables_build(C.byref(m), C.byref(h)) == 1
    assert b"dimension" in lib.rtmc_last_error(None)
    # knots must be strictly increasing
    c = np.array([0.0, 0.5, 0.5, 1.0])
    t = np.array([0.0, 1.0, 2.0, 3.0])
    nk = (C.c_int64 * 1)(4)
    cp = (C.POINTER(C.c_double) * 1)(_lib.dptr(c))
    tp = (C.POINTER(C.c_double) * 1)(_lib.dptr(t))
    assert lib.rtmc_tables_from_knots(1, nk, cp, tp, C.byref(h)) == 5
    assert b"strictly increasing" in lib.rtmc_last_error(None)
    # forward with a NULL problem is an argument error, not a crash
    assert lib.rtmc_forward(None, None, None, None, None) == 1
    assert lib.rtmc_forward_noalloc(None, None, None, None, None) == 1


def test_tables_from_knots_roundtrip_and_eval():
    c = np.array([0.0, 0.25, 0.5, 1.0])
    t = np.array([0.0, 1.0, 1.5, 3.0])
    T = _lib.Tables.from_knots([(c, t)])
    cc, tt = T.knots(0)
    assert np.array_equal(cc, c) and np.array_equal(tt, t)
    # griddedInterpolant: linear inside, linear extrapolation outside
    u = np.array([-0.1, 0.0, 0.125, 0.75, 1.0, 1.2])
    assert np.allclose(T.eval(0, u), [-0.4, 0.0, 0.5, 2.25, 3.0, 3.6])
