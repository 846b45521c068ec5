"""The C-ABI library builds, loads and exports every entry point include/cpd.h
declares; the ctypes structures match the header's layout. No GPU calls."""
import ctypes as C
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "cpd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cpd_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from compound_prism_designer import _native as N

    names = _declared()
    assert len(names) >= 20
    lib = C.CDLL(N.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in N.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


def test_struct_sizes_match_header_layout():
    from compound_prism_designer import _native as N

    # cpd_spectrometer_params: 2 int + 36+7+6+1+2 doubles + 2 x 32-bit + 6+2+2+2 doubles
    assert C.sizeof(N.SpectrometerParams) == 8 + 8 * (36 + 7 + 6 + 3) + 8 + 8 * 12
    assert C.sizeof(N.Fitness) == 6 * 8 + 4 * 8 + 8
    assert C.sizeof(N.BatchItem) == 16
    assert N.lib.cpd_abi_version() == 1


def test_status_strings():
    from compound_prism_designer import _native as N

    assert N.status_string(N.OK) == "OK"
    assert N.status_string(N.RAYTRACE_TOTAL_INTERNAL_REFLECTION) == "TotalInternalReflection"
    assert N.status_string(999) == "Unknown"
