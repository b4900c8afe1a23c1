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
