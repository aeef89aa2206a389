"""The reference-compatible command line (batchgemm_gb300/cli/bgemm_gemm.cpp):
`bgemm_gemm BATCH TLP_thres wavefront_thres` with the reference's shape file
format and log line."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "batchgemm_gb300", "bgemm_gemm")
LINE = re.compile(r"^totalgflops=([0-9.]+)      ==============   ([0-9.]+)$")


def shapes_file(tmp_path, n):
    shp = np.load(os.path.join(ROOT, "tests", "golden", "ref_dataset_shapes.npy"))[:n]
    p = tmp_path / "data_MN_K_512_128"
    p.write_text("".join("%d %d %d\n" % tuple(r) for r in shp))
    return str(p), shp


def test_cli_usage_and_missing_shape_file(built_lib, tmp_path):
    """Argument and input errors are reported like the reference's, before
    any device work (no GPU needed)."""
    r = subprocess.run([EXE], capture_output=True, text=True)
    assert r.returncode != 0 and "Usage: input the batch size" in r.stdout
    r = subprocess.run([EXE, "8", "512", "6000", "--data", str(tmp_path / "none")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "Error opening input" in r.stdout
    short, _ = shapes_file(tmp_path, 4)
    r = subprocess.run([EXE, "8", "512", "6000", "--data", short], capture_output=True, text=True)
    assert r.returncode != 0 and "line 5" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["simt", "tf32x3"])
def test_cli_log_line(cuda, tmp_path, mode):
    """The run.sh sweep's batch sizes give the reference's log line, with the
    reference's flop count sum(2MNK + 2MN)."""
    for batch in (8, 64, 256):
        path, shp = shapes_file(tmp_path, batch)
        r = subprocess.run([EXE, str(batch), "512", "6000", "--data", path, "--mode", mode],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        m = LINE.match(r.stdout.strip().splitlines()[-1])
        assert m, r.stdout
        M, N, K = (shp[:, i].astype(np.float64) for i in range(3))
        want = float(np.sum(2 * M * N * K + 2 * M * N) / 1e9)
        assert abs(float(m.group(1)) - want) <= 1e-6 * max(1.0, want)
        assert float(m.group(2)) > 0
