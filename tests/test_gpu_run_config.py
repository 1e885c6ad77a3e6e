"""`geodesic run config.toml` with `backend = "cuda"` (needs a GPU): the run
loop of `geodesic_cuda.run` on the device, from AMBER files through the
config to the DCD and CSV files.

* A single system with H bonds constrained follows the oracle's run of the
  same files (mixed precision, 30 steps of 2 fs: every float32 coordinate
  within 1e-4 A, energies within the CSV's three decimals plus 1e-4
  relative), and two runs of the same config write byte-identical files
  (geodesic/tests/determinism.rs:66-84).
* A `[[system]]` batch of unconstrained systems writes, for each system, the
  DCD that the system's own single-system config writes, byte for byte (a
  batch reproduces each system's run bit for bit), and energies that agree
  to the CSV's precision."""
import os
import shutil
import sys

import numpy as np
import pytest

from geodesic_cuda import run

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_fixtures import read_dcd  # noqa: E402
from test_run_config import oracle_expected, write_case  # noqa: E402

pytestmark = pytest.mark.gpu


def csv_columns(path):
    rows = [r.split(",") for r in open(path).read().splitlines()[1:]]
    return np.array([[float(x) for x in r] for r in rows])


def test_config_run_follows_oracle_and_reruns_bit_identical(tmp_path):
    cfg = write_case(tmp_path, [("sys", 600, 61, 0.3)], 30, 5, frames_per_batch=4)
    first = run.run_from_config_file(cfg)
    dcd_bytes = (tmp_path / "traj.dcd").read_bytes()
    csv_text = (tmp_path / "energy.csv").read_text()
    again = run.run_from_config_file(cfg)
    assert (tmp_path / "traj.dcd").read_bytes() == dcd_bytes
    assert (tmp_path / "energy.csv").read_text() == csv_text
    assert first == again and first.n_frames == 7

    n, frames, pot, kin = oracle_expected(tmp_path, "sys", 30, 5)
    header, dcd = read_dcd(tmp_path / "traj.dcd")
    assert header["nset"] == len(frames) == 7 and header["natom"] == n
    assert np.abs(dcd.astype(np.float64) - frames).max() < 1e-4
    cols = csv_columns(tmp_path / "energy.csv")
    assert np.array_equal(cols[:, 0], np.arange(0, 31, 5))
    assert np.allclose(cols[:, 2], pot, rtol=1e-4, atol=1e-3), (cols[:, 2], pot)
    assert np.allclose(cols[:, 3], kin, rtol=1e-4, atol=1e-3), (cols[:, 3], kin)


def test_batch_config_writes_each_systems_own_run(tmp_path):
    systems = [("a", 500, 62, 0.0), ("b", 800, 63, 0.0), ("c", 350, 64, 0.0)]
    cfg = write_case(tmp_path, systems, 30, 10, constrain=False)
    out = run.run_from_config_file(cfg)
    assert [s.name for s in out] == ["a", "b", "c"] and [s.n_frames for s in out] == [4, 4, 4]
    for (name, _, _, _), s in zip(systems, out):
        alone = tmp_path / f"{name}_alone"
        alone.mkdir()
        for ext in ("prmtop", "inpcrd"):
            shutil.copy(tmp_path / f"{name}.{ext}", alone / f"{name}.{ext}")
        one_cfg = write_case(alone, None, 30, 10, constrain=False, files=[(name, f"{name}.prmtop", f"{name}.inpcrd")])
        one = run.run_from_config_file(one_cfg)
        assert (tmp_path / f"traj_{name}.dcd").read_bytes() == (alone / "traj.dcd").read_bytes(), name
        a, b = csv_columns(tmp_path / f"energy_{name}.csv"), csv_columns(alone / "energy.csv")
        assert np.array_equal(a[:, :2], b[:, :2]) and np.allclose(a[:, 2:], b[:, 2:], rtol=1e-6, atol=2e-3), name
        assert abs(s.final_potential - one.final_potential) <= 1e-6 * max(1.0, abs(one.final_potential))
