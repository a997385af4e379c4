"""The C-ABI library loads and exports every symbol the public header
declares (no compute calls: no GPU needed)."""
import ctypes
import os

import pytest

import jubik_gb300 as ju
from jubik_gb300 import _lib


def _built():
    return os.path.exists(_lib.LIB_PATH)


@pytest.mark.skipif(not _built(), reason="library not built")
def test_library_exports_every_header_symbol():
    lib = _lib.load()
    names = _lib.header_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    # and the ctypes signature table covers exactly the header
    assert sorted(_lib._SIGS) == names


@pytest.mark.skipif(not _built(), reason="library not built")
def test_info_calls_need_no_gpu():
    lib = _lib.load()
    assert lib.jubik_abi_version() == 1
    assert lib.jubik_fused_supported(192, _lib.F32) == 1
    assert lib.jubik_fused_supported(192, _lib.F64) == 0
    assert lib.jubik_fused_supported(80, _lib.F32) == 0
    assert lib.jubik_fused_supported(160, _lib.F32) == 1
    assert lib.jubik_fused_supported(160, _lib.F64) == 0
    assert lib.jubik_fft_length_supported(1134) == 1  # 2 . 9 . 9 . 7
    assert lib.jubik_fft_length_supported(96) == 1
    assert lib.jubik_fft_length_supported(131) == 0  # prime > 64


@pytest.mark.skipif(not _built(), reason="library not built")
def test_invalid_plan_descriptions_fail_without_touching_the_gpu():
    lib = _lib.load()
    h = ctypes.c_void_p()
    bad = [
        _lib.PlanDesc(1, 1, 64, 64, 4, 0, 0, 0, 1.0),     # margin 0: reference crops [0:-0]
        _lib.PlanDesc(1, 1, 64, 64, 0, 4, 0, 0, 1.0),     # no patches
        _lib.PlanDesc(1, 1, 64, 32, 4, 4, 0, 0, 1.0),     # non-square stride
        _lib.PlanDesc(1, 1, 64, 64, 4, 4, 7, 0, 1.0),     # bad dtype
    ]
    for d in bad:
        st = lib.jubik_plan_create(ctypes.byref(d), ctypes.byref(h))
        assert st == _lib.ERR_INVALID_ARGUMENT, _lib.last_error()
        assert h.value is None
    with pytest.raises(ValueError):
        _lib.check(_lib.ERR_INVALID_ARGUMENT, "x")
    with pytest.raises(_lib.JubikUnsupported):
        _lib.check(_lib.ERR_UNSUPPORTED, "x")


def test_header_parser_finds_declarations():
    names = _lib.header_symbols()
    assert "jubik_poisson_energy_grad" in names and "jubik_plan_create" in names


@pytest.mark.skipif(not _built(), reason="library not built")
def test_group_and_cf_argument_errors_without_a_gpu():
    """Argument checks of the grouped-launch and correlated-field entries run
    before any CUDA call."""
    lib = _lib.load()
    g = ctypes.c_void_p()
    assert lib.jubik_group_create(None, 0, ctypes.byref(g)) == _lib.ERR_INVALID_ARGUMENT
    plans = (ctypes.c_void_p * 2)(None, None)
    assert lib.jubik_group_create(plans, 2, ctypes.byref(g)) == _lib.ERR_INVALID_ARGUMENT
    assert "NULL" in _lib.last_error()
    cf = ctypes.c_void_p()
    pidx = (ctypes.c_int32 * 16)(*([0] * 15 + [3]))
    # pindex value outside [0, n_modes)
    assert lib.jubik_cf_create(1, 4, 4, pidx, 3, _lib.F32, ctypes.byref(cf)) == \
        _lib.ERR_INVALID_ARGUMENT
    assert "pindex" in _lib.last_error()
    # five fields (at most four), a bad dtype, a prime factor above the FFT radix limit
    assert lib.jubik_cf_create(5, 4, 4, pidx, 4, _lib.F32, ctypes.byref(cf)) == \
        _lib.ERR_INVALID_ARGUMENT
    assert lib.jubik_cf_create(1, 4, 4, pidx, 4, 9, ctypes.byref(cf)) == \
        _lib.ERR_INVALID_ARGUMENT
    big = (ctypes.c_int32 * (4 * 67))()
    assert lib.jubik_cf_create(1, 4, 67, big, 1, _lib.F32, ctypes.byref(cf)) == \
        _lib.ERR_UNSUPPORTED
    assert cf.value is None
    assert lib.jubik_cf_apply(None, None, None, None, None, None, 0, 0, 0, None, None) == \
        _lib.ERR_INVALID_ARGUMENT
    assert lib.jubik_cf_destroy(None) == _lib.OK


@pytest.mark.skipif(not _built(), reason="library not built")
def test_convolve2d_argument_errors_without_a_gpu():
    """Both convolution entries reject an unknown dtype, and the allocation-free
    one rejects plane counts whose scratch would overflow, before any CUDA call."""
    lib = _lib.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the checks run first
    for name in ("jubik_convolve2d", "jubik_convolve2d_noalloc"):
        fn = getattr(lib, name)
        assert fn(dummy, 1, dummy, 1, 8, 8, 1.0, 5, dummy, None) == _lib.ERR_INVALID_ARGUMENT
        assert "dtype" in _lib.last_error() or "invalid" in _lib.last_error()
    huge = 1 << 62  # bk * h * w * 16 would wrap around 2^64
    assert lib.jubik_convolve2d_noalloc(dummy, huge, dummy, huge, 64, 64, 1.0, _lib.F64, dummy,
                                        None) == _lib.ERR_INVALID_ARGUMENT
    assert "exceed" in _lib.last_error()


@pytest.mark.skipif(not _built(), reason="library not built")
def test_psf_interpolate_argument_errors_without_a_gpu():
    """The PSF interpolator rejects bad layouts, fields and too many radii before any
    CUDA call."""
    lib = _lib.load()
    d = out = ctypes.c_void_p(16)  # never dereferenced: the checks run first
    fn = lib.jubik_psf_interpolate
    ok = dict(E=1, R=3, h=16, w=16, nx=64, ny=64, npatch=4, layout=0, dtype=_lib.F64)

    def call(**kw):
        k = dict(ok, **kw)
        return fn(d, d, d, d, d, k["E"], k["R"], k["h"], k["w"], k["nx"], k["ny"],
                  1.0, 1.0, k["npatch"], k["layout"], k["dtype"], out, None)

    assert call(layout=7) == _lib.ERR_INVALID_ARGUMENT
    assert call(nx=62) == _lib.ERR_INVALID_ARGUMENT
    assert call(R=2049) == _lib.ERR_INVALID_ARGUMENT
    assert "radii" in _lib.last_error()
