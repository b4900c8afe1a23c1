"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares (no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(steps_gpu_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import steps_gb300 as S
    if not os.path.exists(S.LIB_PATH):
        from steps_gb300 import build
        build.build()
    return S.load_library()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "steps_gpu_forces" in names and "steps_gpu_init" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_calls_without_init_fail_cleanly(lib):
    # Before steps_gpu_init every entry point reports STEPS_E_STATE (2) and a message.
    import steps_gb300 as S
    if lib.steps_gpu_launch_count() != 0:
        pytest.skip("library already initialised in this process")
    rc = lib.steps_gpu_set_particles(4, None, None)
    assert rc == S.STEPS_E_STATE
    assert b"steps_gpu_init" in lib.steps_gpu_error_string()
    assert lib.steps_gpu_abi_version() == 1


def test_missing_library_fails_loudly(tmp_path):
    """No CPU fallback: without the built library the package raises."""
    import steps_gb300 as S

    loaded, S._LIB = S._LIB, None
    try:
        with pytest.raises(RuntimeError, match="is missing"):
            S.load_library(str(tmp_path / "libsteps_gb300.so"))
    finally:
        S._LIB = loaded


def test_header_is_plain_c_and_links(tmp_path, lib):
    """include/steps_gb300.h compiles as strict C99 and a C program that takes
    the address of every declared entry point links against the library with
    no unresolved symbol (the boundary needs no C++ on the caller's side)."""
    import subprocess

    names = declared_symbols()
    src = tmp_path / "use_abi.c"
    body = "\n".join(f"    (void (*)(void))&{n}," for n in names)
    src.write_text('#include "steps_gb300.h"\n#include <stdio.h>\n'
                   f"static void (*const entry_points[])(void) = {{\n{body}\n}};\n"
                   "int main(void) { printf(\"%d\\n\", (int)(sizeof entry_points / sizeof *entry_points)); "
                   "return 0; }\n")
    exe = tmp_path / "use_abi"
    lib_dir = os.path.join(ROOT, "steps_gb300", "_build")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", lib_dir, "-lsteps_gb300",
                        "-Wl,--no-undefined"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_bounds_checked_library_exports_the_same_symbols(lib):
    """The -DSTEPS_CHECK build is the same C-ABI; only it reports checks
    compiled in (nothing that touches the GPU is called)."""
    import steps_gb300 as S

    if not os.path.exists(S.CHECK_LIB_PATH):
        from steps_gb300 import build
        build.build()
    chk = ctypes.CDLL(S.CHECK_LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(chk, n)]
    assert not missing, f"not exported by the checked build: {missing}"
    assert chk.steps_gpu_checks_compiled() == 1
    assert lib.steps_gpu_checks_compiled() == 0
