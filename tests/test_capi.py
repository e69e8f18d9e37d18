"""CPU tests of the C ABI: the library builds for sm_103a, loads, and exports every declared symbol.
No compute call is made without a GPU."""
import ctypes
import subprocess

from luisacompute_gb300 import _capi


def test_exports_every_declared_symbol(lcx):
    declared = _capi.declared_symbols()
    assert len(declared) >= 16
    out = subprocess.run(["nm", "-D", "--defined-only", str(_capi.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        assert hasattr(lcx, s)


def test_version_and_error_string(lcx):
    assert lcx.lcx_version() == 0x000100
    assert lcx.lcx_last_error_string() is not None


def test_struct_sizes():
    assert ctypes.sizeof(_capi.LcxAccelOption) == 8
    assert ctypes.sizeof(_capi.LcxMeshBuildCommand) == 64
    assert ctypes.sizeof(_capi.LcxAccelStats) == 56
    assert ctypes.sizeof(_capi.LcxPtStats) == 32


def test_tuning_knobs_round_trip_and_range_checks(lcx):
    """Every knob the autotuner sets is host state: settable, readable and range-checked
    without a GPU."""
    from luisacompute_gb300 import autotune as A
    old = A.current()
    try:
        cfg = A.Config(leaf_max=3, width=4, blas_cube=0, refill=16, short_stack=24, mode=1, reorder_bits=7,
                       postpone=12, split=1.0, blas_sah=0, collapse=0)
        A.apply(cfg)
        assert A.current() == cfg
        assert lcx.lcx_set_trace_stack(12) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_trace_reorder(10, 0) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_build_tuning(4, 8) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_build_tuning(2, 9) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_build_morton(2, 0, 0) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_trace_tuning(0, 0, 0) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_trace_tuning(4, 0, 4) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_build_split(ctypes.c_float(-1.0)) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_build_blas_sah(2) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_build_collapse(2) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_set_build_tlas_sah(2) == _capi.LCX_ERR_INVALID_ARG
        assert A.current() == cfg  # rejected calls change nothing
    finally:
        A.apply(old)
    assert A.current() == old


def test_step_bound_knob(lcx):
    """The per-ray step bound is host state: default 2^22, settable, 0 restores the default,
    larger values are rejected."""
    v = ctypes.c_uint32(0)
    assert lcx.lcx_get_trace_step_bound(ctypes.byref(v)) == 0 and v.value == 1 << 22
    try:
        assert lcx.lcx_set_trace_step_bound(5) == 0
        assert lcx.lcx_get_trace_step_bound(ctypes.byref(v)) == 0 and v.value == 5
        assert lcx.lcx_set_trace_step_bound((1 << 22) + 1) == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_get_trace_step_bound(ctypes.byref(v)) == 0 and v.value == 5
    finally:
        assert lcx.lcx_set_trace_step_bound(0) == 0
    assert lcx.lcx_get_trace_step_bound(ctypes.byref(v)) == 0 and v.value == 1 << 22
