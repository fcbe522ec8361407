"""The C ABI library loads and exports every entry point include/sf_capi.h
declares; argument validation and the no-GPU path work without a device."""

import ctypes
import os
import re

import numpy as np
import pytest

from sph_seepage_flows_gb300 import build, capi, scenes


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return capi.load()


def test_exports_every_declared_symbol(lib):
    names = capi.header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    out = os.popen(f"nm -D --defined-only {capi.LIB_PATH}").read()
    exported = set(re.findall(r" T (sf_\w+)", out))
    assert set(names) <= exported


def test_version_and_header_version(lib):
    assert b"sm_103a" in lib.sf_version()
    text = open(capi.HEADER).read()
    assert int(re.search(r"#define SF_CAPI_VERSION (\d+)", text).group(1)) == lib.sf_capi_version()


def test_null_and_bad_arguments_are_rejected(lib):
    h = ctypes.c_void_p()
    assert lib.sf_create(None, None, None, None, 0, None, ctypes.byref(h)) == 1
    assert lib.sf_destroy(None) == 1
    assert lib.sf_step(None, 0.01, None, None) == 1
    assert lib.sf_get_field(None, 0, 0, 0, None, 0, 0) == 1


def test_invalid_scene_is_rejected_before_device_use(lib):
    sc = scenes.tiny()
    sc.label = sc.label.copy()
    sc.label[0] = 7
    with pytest.raises(capi.SfError) as e:
        capi.Simulation(sc)
    assert e.value.status == 1 and "labels" in str(e.value)
    sc = scenes.tiny()
    with pytest.raises(capi.SfError) as e:
        capi.Simulation(sc, capacity=sc.n - 1)
    assert e.value.status == 1


def test_create_without_device_reports_no_device(lib):
    if lib.sf_device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(capi.SfError) as e:
        capi.Simulation(scenes.tiny())
    assert e.value.status == 5


def test_header_is_plain_c(tmp_path):
    """include/sf_capi.h is a C interface: it compiles as strict C99 and as
    C++17 with no warnings."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "use.c"
    src.write_text('#include "sf_capi.h"\nint main(void) { return SF_CAPI_VERSION > 0 ? 0 : 1; }\n')
    for cmd in ([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only"],
                [shutil.which("g++") or "g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c++"]):
        r = subprocess.run(cmd + ["-I", os.path.join(root, "include"), str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
