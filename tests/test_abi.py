"""The C-ABI library loads and exports every symbol include/msfec_cuda.h declares."""
import ctypes
import os
import re


REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(REPO, "include", "msfec_cuda.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(msfec_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_expected_api():
    import msfec
    assert sorted(msfec.EXPORTED) == declared_functions()


def test_library_exports_every_declared_symbol():
    import msfec_build
    lib = msfec_build.build()
    L = ctypes.CDLL(lib)
    for name in declared_functions():
        assert hasattr(L, name), name


def test_status_strings_and_defaults_without_gpu():
    import msfec
    L = msfec.load_library()
    cfg = msfec.Config()
    L.msfec_config_default(ctypes.byref(cfg))
    assert cfg.precision == msfec.PRECISION_MIXED and cfg.rtol == 1e-12 and cfg.max_refine >= 1
    for s in range(8):
        assert L.msfec_status_string(s)
    # argument checks happen before any device work
    assert L.msfec_create(None, None) == msfec.ERROR_INVALID_ARGUMENT


def test_header_is_plain_c():
    """The boundary is a C ABI: the header compiles as strict C99 (no C++ or
    torch types), so cgo / ctypes / JNI bindings can include it directly."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-x", "c",
                        os.path.join(REPO, "include", "msfec_cuda.h")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
