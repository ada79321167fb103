"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/inspire_gpu.h (no compute call: this runs without a GPU)."""
import ctypes
import subprocess

import pytest


@pytest.fixture(scope="module")
def lib_path():
    import build_lib

    return build_lib.build()


def test_library_exports_every_declared_symbol(lib_path):
    from inspire import _native

    declared = _native.declared_symbols()
    assert len(declared) >= 19
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert set(declared) <= exported


def test_binding_covers_header(lib_path):
    from inspire import _native

    L = _native.load(lib_path)
    for s in _native.declared_symbols():
        assert getattr(L, s).argtypes is not None, s  # every declared entry point has a signature
    assert L.inspire_version().decode().startswith("inspire-gb300")


def test_missing_library_fails_loudly(tmp_path):
    from inspire import _native

    saved = _native._lib
    _native._lib = None
    try:
        with pytest.raises(OSError, match="not built"):
            _native.load(str(tmp_path / "nope.so"))
    finally:
        _native._lib = saved


def test_params_validation_mirrors_reference():
    """InspireParams::validate (params.rs:348-387) on the host side."""
    from inspire import InspireParams

    p = InspireParams.secure_128_d2048()
    p.validate()
    assert p.gadget_len == 3 and p.q == 268369921 * 249561089
    assert p.delta() == p.q // 65537
    bad = InspireParams(ring_dim=2048, crt_moduli=(268369921, 268369921))
    with pytest.raises(ValueError, match="coprime"):
        bad.validate()
    with pytest.raises(ValueError, match="power of two"):
        InspireParams(ring_dim=1000).validate()
