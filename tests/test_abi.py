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


def test_config_ranges_rejected_without_gpu():
    """Out-of-range configuration fields are rejected by msfec_create before any
    device work (MSFEC_ERROR_INVALID_ARGUMENT)."""
    import msfec
    L = msfec.load_library()
    bad = [("nedrt_zt_place", 3), ("nedrt_zt_place", -1), ("nedrt_inner_rtol", -1e-6), ("nedrt_inner_rtol", 1.0),
           ("nedrt_ctas_per_sm", 3), ("nedrt_stage", 2), ("nedrt_precond", 3), ("inner_rtol", 0.0)]
    for field, value in bad:
        cfg = msfec.Config()
        L.msfec_config_default(ctypes.byref(cfg))
        setattr(cfg, field, value)
        h = ctypes.c_void_p()
        assert L.msfec_create(ctypes.byref(h), ctypes.byref(cfg)) == msfec.ERROR_INVALID_ARGUMENT, (field, value)
    cfg = msfec.Config()
    L.msfec_config_default(ctypes.byref(cfg))
    assert cfg.nedrt_inner_rtol == 3e-6 and cfg.nedrt_zt_place == 0 and cfg.inner_rtol == 1e-6


def test_ctypes_config_matches_c_layout(tmp_path):
    """The ctypes view of msfec_config has the C struct's size and field
    offsets (gcc on the header)."""
    import shutil
    import subprocess
    import pytest
    import msfec
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = [f[0] for f in msfec.Config._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "msfec_cuda.h"\nint main(void) {\n'
                   '  printf("%zu\\n", sizeof(msfec_config));\n' +
                   "".join(f'  printf("%zu\\n", offsetof(msfec_config, {n}));\n' for n in names) + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert out[0] == ctypes.sizeof(msfec.Config)
    for n, off in zip(names, out[1:]):
        assert getattr(msfec.Config, n).offset == off, n
