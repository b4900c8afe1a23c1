"""The bounds-checked build (libsteps_gb300_check.so, -DSTEPS_CHECK).

Its kernels compare every tile, chunk, slot, output-row, table-cell and
ordering index with its bound and record the first one out of range; the
call then returns STEPS_E_BOUNDS. The edge-size and planted-pair cases of
the other GPU tests run once more in a child process on that library: they
must pass with no index out of range. The mechanism itself is checked with
the self-test entry point, which submits an index against the bound 16
without dereferencing it.
"""
import os
import re
import subprocess
import sys

import pytest

import steps_gb300 as S

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = [
    "tests/test_gpu_r3.py::test_edge_sizes",
    "tests/test_gpu_r3.py::test_coincident_and_softened_pairs",
    "tests/test_gpu_r3.py::test_shapes_agree",
    "tests/test_gpu_r3.py::test_packed_fp32x2_variant",
    "tests/test_gpu_r3.py::test_empty_range",
    "tests/test_gpu_r3.py::test_resident_forces_range",
    "tests/test_gpu_periodic.py::test_periodic_edge_sizes",
    "tests/test_gpu_periodic.py::test_t3_fp64",
    "tests/test_gpu_periodic.py::test_t3_nearest_image_at_half_box",
    "tests/test_gpu_periodic.py::test_t3_mixed_shapes_and_workload_table",
    "tests/test_gpu_periodic.py::test_s1r2_table_fp64",
    "tests/test_gpu_periodic.py::test_s1r2_table_mixed",
    "tests/test_gpu_periodic.py::test_s1r2_images_mixed",
    "tests/test_gpu_periodic.py::test_s1r2_background_terms",
    "tests/test_gpu_periodic.py::test_s1r2_nearest_image_at_half_period",
    "tests/test_gpu_periodic.py::test_s1r2_ngp_at_cell_faces",
    "tests/test_gpu_batch.py::test_batch_graph_and_plain_match_oracle",
    "tests/test_gpu_kdk.py::test_kdk_periodic_wrap",
    "tests/test_gpu_check.py::test_bounds_check_self_test",
]


def test_bounds_check_self_test(engine):
    if not engine.checks_compiled():
        rc, msg = engine.test_bounds_check(16)
        assert rc == S.STEPS_E_STATE, (rc, msg)
        return
    for index in (16, -1, 1 << 20):
        rc, msg = engine.test_bounds_check(index)
        assert rc == S.STEPS_E_BOUNDS, (index, rc, msg)
        assert "self-test index" in msg and f"{index} outside [0, 16)" in msg, msg
    for index in (0, 5, 15):
        assert engine.test_bounds_check(index) == (S.STEPS_OK, ""), index
    # the record is cleared once reported: the next call is clean
    from steps_gb300 import workloads as W

    ps = W.r3_compactified(300, 480.0, seed=3, displace=True)
    engine.set_particles(ps.m, ps.eps)
    engine.forces(ps.x, S.params(S.R3), S.MIXED)


@pytest.mark.skipif(os.environ.get("STEPS_GB300_LIB") == S.CHECK_LIB_PATH,
                    reason="already running on the bounds-checked library")
def test_edge_and_planted_cases_under_bounds_checks():
    assert os.path.exists(S.CHECK_LIB_PATH), "build() makes the bounds-checked library"
    env = dict(os.environ, STEPS_GB300_LIB=S.CHECK_LIB_PATH, STEPS_GB300_QUIET="1")
    cmd = [sys.executable, "-m", "pytest", "-q", "-m", "gpu", "-p", "no:cacheprovider"]
    listed = subprocess.run(cmd + ["--collect-only", *CASES], cwd=ROOT, env=env, capture_output=True, text=True)
    collected = int(re.search(r"(\d+) tests? collected", listed.stdout).group(1))
    assert collected >= len(CASES), listed.stdout[-2000:]
    r = subprocess.run(cmd + ["-x", *CASES], cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    m = re.search(r"(\d+) passed", r.stdout)
    assert m and int(m.group(1)) == collected and "failed" not in r.stdout, r.stdout[-2000:]
