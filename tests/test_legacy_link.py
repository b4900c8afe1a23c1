"""Link check of the drop-in: the reference's own driver-side translation
units (StePS/src/step.cc, utils.cc, ewald_space.cc, friedmann_solver.cc),
compiled unmodified from the reference tree, link against
steps_gb300/legacy/forces_gb300.cc + libsteps_gb300.so with no unresolved
symbol, for each topology switch set. Runs where the reference tree is
present (nothing is executed: no GPU needed)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ref_src():
    """The reference source directory oracle/Makefile's `ref` target was built
    from (it records it in oracle/_ref/ref_src.txt); "" when not built here."""
    try:
        with open(os.path.join(ROOT, "oracle", "_ref", "ref_src.txt")) as f:
            return f.read().strip()
    except OSError:
        return ""


REF_SRC = _ref_src()
LIB_DIR = os.path.join(ROOT, "steps_gb300", "_build")

VARIANTS = {
    "r3": [],
    "t3": ["-DPERIODIC", "-DEWALD_INTERPOLATION_ORDER=4"],
    "s1nl": ["-DPERIODIC_Z", "-DPERIODIC_Z_NOLOOKUP"],
    "s1tab": ["-DPERIODIC_Z", "-DEWALD_INTERPOLATION_ORDER=2"],
}


@pytest.mark.skipif(not REF_SRC or not os.path.isdir(REF_SRC), reason="reference tree not present")
@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_reference_driver_links_with_shim(tmp_path, variant):
    if not os.path.exists(os.path.join(LIB_DIR, "libsteps_gb300.so")):
        from steps_gb300 import build
        build.build()
    flags = ["-std=gnu++17", "-O1", "-fPIC", "-fopenmp", "-include", "cstring", "-I", os.path.join(ROOT, "oracle",
             "mpi_stub"), "-I", REF_SRC, "-I", os.path.join(ROOT, "include"), "-DCOSMOPARAM=0", "-DSTEPS_HARNESS_NO_SOFTENING_PROBE", "-w"] + VARIANTS[variant]
    objs = []
    for tu in ("step", "utils", "ewald_space", "friedmann_solver"):
        o = tmp_path / f"{tu}.o"
        subprocess.run(["g++"] + flags + ["-c", os.path.join(REF_SRC, tu + ".cc"), "-o", str(o)], check=True)
        objs.append(str(o))
    for src in (os.path.join(ROOT, "steps_gb300", "legacy", "forces_gb300.cc"),
                os.path.join(ROOT, "oracle", "ref_harness.cc")):
        o = tmp_path / (os.path.basename(src) + ".o")
        subprocess.run(["g++"] + flags + ["-c", src, "-o", str(o)], check=True)
        objs.append(str(o))
    out = tmp_path / f"libdriver_{variant}.so"
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-o", str(out)] + objs +
                       ["-L", LIB_DIR, "-lsteps_gb300", "-Wl,--no-undefined", "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
