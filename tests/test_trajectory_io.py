"""Trajectory writers against the reference's files (CPU only).

The DCD writer, given the 100 frames decoded from the reference's golden
trajectory (geodesic/tests/golden/ala_dipeptide_ref.dcd, written by
geodesic-io/src/dcd.rs at 1 fs, every step), reproduces that file byte for
byte: same size and SHA-256 (both recorded by tests/golden/make_fixtures.py).
The energy CSV follows geodesic-io/src/export.rs:18-51."""
import hashlib
import json
import os

import numpy as np

from geodesic_cuda import trajectory

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_dcd_writer_reproduces_the_reference_file(tmp_path):
    frames = np.load(os.path.join(GOLDEN, "ala_dipeptide_ref_frames.npy"))
    with open(os.path.join(GOLDEN, "ala_dipeptide_ref_header.json")) as f:
        ref = json.load(f)
    path = tmp_path / "t.dcd"
    with trajectory.DcdWriter(path, ref["natom"], ref["nsavc"], 0.001) as w:
        w.write_frames(frames)
    raw = path.read_bytes()
    assert len(raw) == ref["file_bytes"]
    assert hashlib.sha256(raw).hexdigest() == ref["file_sha256"]


def test_dcd_writer_patches_the_frame_count_and_checks_rows(tmp_path):
    path = tmp_path / "t.dcd"
    w = trajectory.DcdWriter(path, 3, 10, 0.002)
    w.write_frame(np.arange(3), np.arange(3) + 1.0, np.arange(3) + 2.0)
    w.write_frame(np.zeros(3), np.zeros(3), np.zeros(3))
    try:
        w.write_frame(np.zeros(4), np.zeros(3), np.zeros(3))
        raise AssertionError("a row of the wrong length was accepted")
    except ValueError:
        pass
    w.close()
    raw = path.read_bytes()
    assert int.from_bytes(raw[8:12], "little") == 2               # NSET
    assert int.from_bytes(raw[16:20], "little") == 10             # NSAVC
    assert np.frombuffer(raw[44:48], "<f4")[0] == np.float32(0.002 * 20.455)  # DELTA (AKMA)
    assert len(raw) == (8 + 84) + (8 + 84) + (8 + 4) + 2 * 3 * (8 + 12)


def test_energy_log_format(tmp_path):
    path = tmp_path / "e.csv"
    with trajectory.EnergyLogWriter(path, 100) as w:
        w.write_row(0, 0.0, -1234.56789, 45.6789)
        w.write_row(500, 1.0, -1200.0, 50.0)
    lines = path.read_text().splitlines()
    assert lines[0] == "step,time_ps,potential_kcal,kinetic_kcal,total_kcal,temperature_K"
    t = 2.0 * 45.6789 / (3.0 * 100 * 0.0019872041)
    assert lines[1] == f"0,0.000,-1234.568,45.679,{-1234.56789 + 45.6789:.3f},{t:.2f}"
    assert lines[2].startswith("500,1.000,-1200.000,50.000,-1150.000,")
