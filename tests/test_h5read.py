"""The HDF5 reader behind steps_gpu_load_table_*_hdf5 (no GPU): the table
fixtures in the reference's table-file layout (tests/golden/make_h5_tables.py,
from the reference's own tables) read back bit for bit; a file written by the
HDF5 library itself -- the reference's example initial conditions -- read where
the reference tree is present; and the errors it reports."""
import os

import numpy as np
import pytest

import steps_gb300 as S
from helpers import GOLDEN, golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ref_example():
    """The reference's example initial conditions (StePS_IC/examples), located
    from the reference source directory the oracle build recorded."""
    try:
        with open(os.path.join(ROOT, "oracle", "_ref", "ref_src.txt")) as f:
            src = f.read().strip()
    except OSError:
        return None
    p = os.path.join(os.path.dirname(os.path.dirname(src)), "StePS_IC", "examples", "Glass_cylindrical_L100_D500.hdf5")
    return p if os.path.exists(p) else None


def test_t3_table_files():
    g = golden("t3_o2")
    ng = int(g["ngrid"])
    t = S.h5_read(os.path.join(GOLDEN, "t3_table_ng17.h5"), "/t3_ewald/T3_EWALD_FORCE_TABLE")
    assert t.shape == (ng, ng, ng, 3) and np.array_equal(t.ravel(), g["table"])
    t = S.h5_read(os.path.join(GOLDEN, "t3_table_ng17_f32.h5"), "/t3_ewald/T3_EWALD_FORCE_TABLE")
    assert np.array_equal(t.ravel(), np.float32(g["table"]).astype(np.float64))


def test_s1r2_table_file():
    g = golden("s1r2_table_o2")
    t = S.h5_read(os.path.join(GOLDEN, "s1r2_table.h5"), "/s1r2_ewald/S1R2_EWALD_FORCE_TABLE")
    assert t.shape == (int(g["shape"][0]), int(g["shape"][1]), 2) and np.array_equal(t.ravel(), g["table"])


@pytest.mark.skipif(_ref_example() is None, reason="reference tree not present")
def test_file_written_by_the_hdf5_library():
    path = _ref_example()
    ids = S.h5_read(path, "/PartType1/ParticleIDs")
    x = S.h5_read(path, "/PartType1/Coordinates")
    m = S.h5_read(path, "/PartType1/Masses")
    assert x.shape == (ids.size, 3) and m.shape == ids.shape
    assert np.array_equal(np.sort(ids), np.arange(ids.size))  # the IDs are 0 .. N-1
    assert x[:, 2].min() >= 0 and x[:, 2].max() < 100  # a cylinder of L_z = 100 (the file's name)
    assert (m > 0).all()


def test_errors(tmp_path):
    with pytest.raises(S.StepsError) as e:
        S.h5_read(os.path.join(GOLDEN, "t3_table_ng17.h5"), "/t3_ewald/NOPE")
    assert e.value.code == S.STEPS_E_ARG and "no object" in str(e.value)
    with pytest.raises(S.StepsError) as e:
        S.h5_read(os.path.join(GOLDEN, "t3_table_ng17.h5"), "/Header")
    assert "not a dataset" in str(e.value)
    bad = tmp_path / "x.h5"
    bad.write_bytes(b"not hdf5" * 32)
    with pytest.raises(S.StepsError) as e:
        S.h5_read(str(bad), "/t3_ewald/T3_EWALD_FORCE_TABLE")
    assert "not an HDF5 file" in str(e.value)
    with pytest.raises(S.StepsError):
        S.h5_read(str(tmp_path / "missing.h5"), "/a")


_FUZZ = r"""
import os, sys
import numpy as np
sys.path.insert(0, {root!r})
import steps_gb300 as S

src = open({path!r}, "rb").read()
tmp = {tmp!r}
rng = np.random.default_rng(7)
cases = [src[:n] for n in range(0, len(src), max(1, len(src) // 97))]
# the structures: the superblock and first group at the start, the dataset's
# object header and the other groups after the raw data at the end
spans = [(0, min(len(src), 1024)), (max(0, len(src) - 3072), len(src))]
for _ in range(400):  # random bytes of the structures overwritten
    b = bytearray(src)
    for _ in range(int(rng.integers(1, 6))):
        lo, hi = spans[int(rng.integers(0, 2))]
        b[int(rng.integers(lo, hi))] = int(rng.integers(0, 256))
    cases.append(bytes(b))
ok = err = 0
for k, c in enumerate(cases):
    with open(tmp, "wb") as f:
        f.write(c)
    try:
        S.h5_read(tmp, {dataset!r})
        ok += 1
    except S.StepsError:
        err += 1
print("done", ok, err)
"""


@pytest.mark.parametrize("name,dataset", [("t3_table_ng17.h5", "/t3_ewald/T3_EWALD_FORCE_TABLE"),
                                          ("s1r2_table.h5", "/s1r2_ewald/S1R2_EWALD_FORCE_TABLE")])
def test_truncated_and_corrupt_files_fail_cleanly(tmp_path, name, dataset):
    """Truncated files and files with random bytes of their structures
    overwritten either read or return STEPS_E_ARG: the reader never reads
    outside the file (run in a child process, so a crash would show)."""
    import subprocess
    import sys

    code = _FUZZ.format(root=ROOT, path=os.path.join(GOLDEN, name), tmp=str(tmp_path / "f.h5"), dataset=dataset)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().startswith("done"), r.stdout[-2000:]
    ok, err = (int(v) for v in r.stdout.split()[1:3])
    assert err > 150  # the truncations and most corruptions
