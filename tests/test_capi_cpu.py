"""CPU checks of the C ABI: the library loads, exports exactly what
include/mpdata.h declares, and rejects bad calls before touching the GPU."""
import ctypes

import pytest

from advectionhpctester_gb300 import _native


def test_library_exports_every_header_symbol(native_lib):
    declared = _native.header_symbols()
    assert declared, "no declarations parsed from include/mpdata.h"
    for name in declared:
        assert hasattr(native_lib, name), name
    assert sorted(_native.SIGNATURES) == declared


def test_version_and_strerror(native_lib):
    assert b"sm_103a" in native_lib.mpdata_version()
    for code in (0, -1, -2, -3, -4, -5, -6, -7):
        assert native_lib.mpdata_strerror(code)
    assert native_lib.mpdata_strerror(-99) == b"unknown error"


@pytest.mark.parametrize("grid,code", [
    ((0, 4, 4, 1, 1, 1, 1), -1),     # empty axis
    ((1, 4, 4, 1, 0, 1, 1), -1),     # open x needs np >= 2
    ((4, 4, 1, 1, 1, 1, 0), -1),     # z wall needs lp >= 2
    ((4, 4, 4, 0, 1, 1, 1), -1),     # halo width 0
    ((4, 4, 4, 1, 2, 1, 1), -1),     # bad boundary flag
    ((4, 4, 70000, 1, 1, 1, 1), -1), # launch geometry limit
])
def test_ws_create_rejects_bad_grid(native_lib, grid, code):
    h = ctypes.c_void_p()
    rc = native_lib.mpdata_ws_create(_native.MpdataGrid(*grid), _native.MpdataOpts(2, 1, 1, 64, 0), h)
    assert rc == code and not h.value


@pytest.mark.parametrize("opts,code", [
    ((0, 1, 1, 64, 0), -2), ((9, 1, 1, 64, 0), -2), ((2, 2, 1, 64, 0), -2),
    ((2, 1, 3, 64, 0), -2), ((2, 1, 1, 16, 0), -2), ((2, 1, 1, 64, 1), -7),
])
def test_ws_create_rejects_bad_opts(native_lib, opts, code):
    h = ctypes.c_void_p()
    rc = native_lib.mpdata_ws_create(_native.MpdataGrid(8, 8, 8, 1, 1, 1, 1), _native.MpdataOpts(*opts), h)
    assert rc == code and not h.value


def test_calls_without_workspace_fail(native_lib):
    assert native_lib.mpdata_ws_destroy(None) == -4
    assert native_lib.mpdata_step_f64(None, *([None] * 9)) == -4
    assert native_lib.mpdata_velprd_f32(None, *([None] * 7), 1.0, 1.0, 1.0, 1.0, 1.0, None, None, None, None) == -4
    out = ctypes.c_int(0)
    assert native_lib.mpdata_ws_error(None, out) == -4


@pytest.mark.parametrize("opt,t_adv,lvertsplit,ipoles,code", [
    (3, 1, 0, 0, -2), (0, 1, 0, 0, -2), (7, 1, 0, 0, -2),   # commented-out or absent CASEs: STOP
    (4, 3, 0, 0, -2), (2, 0, 0, 0, -2), (2, 3, 1, 0, -2),   # bad t_adv under 2/4: STOP, even when split
    (5, 1, 0, 0, -7),                                       # CASE(5): unassociated upwind pointer
    (4, 1, 1, 1, 0), (6, 1, 1, 0, 0),                       # lvertsplit: the split call is commented out
    (2, 1, 0, 0, 0), (2, 2, 0, 0, 0),                       # CASE(2): the mpdata3d call is commented out
    (4, 1, 0, 1, -7)])                                      # ipoles: not on the single-rank path
def test_advec_dwarf_option_dispatch(native_lib, opt, t_adv, lvertsplit, ipoles, code):
    """advec.f90:148-244: the SELECT on legacyoptmode/t_adv STOPs on bad values
    before anything runs; lvertsplit and mode 2 then do nothing; 4 and 6 run
    (not reached here: every array is NULL, so a running mode would fail)."""
    rc = native_lib.mpdata_advec_dwarf_f64(opt, t_adv, 0, lvertsplit, 8, 8, 8, 1, ipoles, 0, 0, 0,
                                           *([None] * 8), 2, 1, None)
    assert rc == code
