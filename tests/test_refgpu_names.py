"""oracle/refgpu.py finds the reference's CUDA kernels in their cubins by
C++ name. The names it builds must be the Itanium-ABI manglings of the
parameter lists StePS/src/forces_cuda.cu declares (:522, :567, :652, :764);
here the host compiler mangles the same declarations. No GPU needed."""
import os
import shutil
import subprocess

import pytest

refgpu = pytest.importorskip("refgpu")

# The reference kernels' parameter lists with REAL spelled out (forces_cuda.cu).
DECLS = """
#include <cstddef>
void ForceKernel(int n, const int N, const R *xx, const R *xy, const R *xz, R *F, const R* M, const R* SOFT_LENGTH,
                 const R mass_in_unit_sphere, const R DE, const int COSMOLOGY, const int COMOVING_INTEGRATION,
                 int ID_min, int ID_max) {}
void ForceKernel_periodic(int n, int N, const R *xx, const R *xy, const R *xz, R *F, const int IS_PERIODIC,
                          const R* M, const R* SOFT_LENGTH, const R L, const R *EwaldTable, int NewaldGrid,
                          int ID_min, int ID_max) {}
void ForceKernel_periodic_z(int n, int N, const R *xx, const R *xy, const R *xz, R *F, const int IS_PERIODIC,
                            const R* M, const R* SOFT_LENGTH, const R L, const R Rsim, const R mass_in_unit_sphere,
                            const R* RADIAL_FORCE_TABLE, const R RADIAL_FORCE_TABLE_SIZE, const R DE,
                            const int COSMOLOGY, const int COMOVING_INTEGRATION, int ID_min, int ID_max) {}
void ForceKernel_periodic_z(int n, const int N, const R *xx, const R *xy, const R *xz, R *F, const int IS_PERIODIC,
                            const R* M, const R* SOFT_LENGTH, const R L, const R Rsim, const R mass_in_unit_sphere,
                            const R* RADIAL_FORCE_TABLE, const int RADIAL_FORCE_TABLE_SIZE, const R* EWALD_TABLE,
                            const size_t EWALD_TABLE_SIZE_RHO, const size_t EWALD_TABLE_SIZE_Z, const R DE,
                            const int COSMOLOGY, const int COMOVING_INTEGRATION, int ID_min, int ID_max) {}
"""


@pytest.mark.parametrize("real,code", [("double", "d"), ("float", "f")])
def test_kernel_names_match_the_declarations(tmp_path, real, code):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "decls.cc"
    src.write_text(f"typedef {real} R;\n" + DECLS)
    obj = tmp_path / "decls.o"
    subprocess.run([cxx, "-c", str(src), "-o", str(obj)], check=True)
    syms = subprocess.run(["nm", str(obj)], check=True, capture_output=True, text=True).stdout
    for topology in ("R3", "T3", "S1", "S1T"):
        assert refgpu.kernel_name(topology, code) in syms, (topology, code)


def test_every_variant_has_a_topology_and_type():
    for v, (topology, code) in refgpu.VARIANTS.items():
        assert topology in ("R3", "T3", "S1", "S1T") and code in ("d", "f"), v
        assert refgpu.cubin_path(v).endswith(f"forces_cuda_{v}.cubin")
        assert os.path.dirname(refgpu.cubin_path(v)) == refgpu.REF_DIR
