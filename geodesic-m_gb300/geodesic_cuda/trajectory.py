"""Trajectory output for device-resident runs: the CHARMM DCD layout and the
energy CSV of the reference's run loop, fed from the frames the device records
during resident steps (`CudaBackend.frames_enable` / `frames_take`).

Formats (the same bytes as the reference's writers, so its readers and tools
take the files unchanged):
* DCD (`geodesic-io/src/dcd.rs:94-136`): an 84-byte header record ("CORD",
  20 control integers: NSET patched on close, ISTART 0, NSAVC = the frame
  interval, NAMNF 0, DELTA = dt in AKMA units as float32, version 24), one
  80-character title line, the atom count, then per frame three float32
  records X, Y, Z; all little-endian with Fortran record markers.
* Energy CSV (`geodesic-io/src/export.rs:18-51`): `step,time_ps,
  potential_kcal,kinetic_kcal,total_kcal,temperature_K`, three decimals
  (two for the temperature), T = 2 KE / (3 N k_B).

`run_with_output` is the run loop of `geodesic/src/lib.rs:284-334` on the
device: the initial frame, then resident steps with a frame every
`frame_interval` steps, drained from the device in batches (no host
synchronisation per frame).
"""
import struct

import numpy as np

AKMA_PER_PS = 20.455               # dcd.rs: 1 AKMA time unit = 1/20.455 ps
KB_KCAL_PER_MOL_K = 0.0019872041   # export.rs: R in kcal/(mol K)
TITLE = b"Created by GEODESIC-M"


def _record(f, payload: bytes):
    n = struct.pack("<i", len(payload))
    f.write(n)
    f.write(payload)
    f.write(n)


class DcdWriter:
    """CHARMM/NAMD-style DCD, single-precision X/Y/Z, no unit-cell block."""

    NSET_OFFSET = 8  # record marker (4) + "CORD" (4): the first control integer

    def __init__(self, path, natom: int, frame_interval: int, dt_ps: float):
        self.path, self.natom, self.n_frames = path, int(natom), 0
        self._f = open(path, "wb")
        ctl = [0] * 20
        ctl[2] = int(frame_interval)                       # NSAVC
        ctl[19] = 24                                       # CHARMM version
        head = bytearray(b"CORD" + struct.pack("<20i", *ctl))
        struct.pack_into("<f", head, 4 + 9 * 4, np.float32(dt_ps * AKMA_PER_PS))  # DELTA
        _record(self._f, bytes(head))
        _record(self._f, struct.pack("<i", 1) + TITLE.ljust(80, b" "))
        _record(self._f, struct.pack("<i", self.natom))

    def write_frame(self, x, y, z):
        for a in (x, y, z):
            a = np.ascontiguousarray(a, dtype="<f4")
            if a.shape != (self.natom,):
                raise ValueError(f"frame row has {a.shape} values, writer expects {self.natom} atoms")
            _record(self._f, a.tobytes())
        self.n_frames += 1

    def write_frames(self, xyz):
        """Frames as a (n_frames, 3, natom) float32 array."""
        for fr in xyz:
            self.write_frame(fr[0], fr[1], fr[2])

    def close(self):
        if self._f is None:
            return
        self._f.seek(self.NSET_OFFSET)
        self._f.write(struct.pack("<i", self.n_frames))
        self._f.close()
        self._f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def temperature_kelvin(kinetic_kcal: float, n_atoms: int) -> float:
    return 2.0 * kinetic_kcal / (3.0 * n_atoms * KB_KCAL_PER_MOL_K)


class EnergyLogWriter:
    """One CSV row per frame, flushed as written."""

    HEADER = "step,time_ps,potential_kcal,kinetic_kcal,total_kcal,temperature_K"

    def __init__(self, path, n_atoms: int):
        self.n_atoms = int(n_atoms)
        self._f = open(path, "w")
        self._f.write(self.HEADER + "\n")
        self._f.flush()

    def write_row(self, step: int, time_ps: float, potential_kcal: float, kinetic_kcal: float):
        total = potential_kcal + kinetic_kcal
        t = temperature_kelvin(kinetic_kcal, self.n_atoms)
        self._f.write(f"{int(step)},{time_ps:.3f},{potential_kcal:.3f},{kinetic_kcal:.3f},{total:.3f},{t:.2f}\n")
        self._f.flush()

    def close(self):
        if self._f is not None:
            self._f.close()
            self._f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_with_output(be, pos, vel, dt_ps: float, n_steps: int, frame_interval: int, dcd_path, csv_path,
                    first_step: int = 0, frames_per_batch: int = 64):
    """Resident BAB steps with trajectory output: the initial frame from the
    given state, then a frame (positions as float32, potential and kinetic
    energy) every `frame_interval` steps, recorded on the device and written
    `frames_per_batch` at a time.  pos/vel ((3, N) float64) end as the final
    state.  Returns the number of frames written."""
    n = be.n
    be.frames_enable(frame_interval, frames_per_batch)
    try:
        with DcdWriter(dcd_path, n, frame_interval, dt_ps) as dcd, EnergyLogWriter(csv_path, n) as csv:
            # frame 0: the state handed in, its forces and energies (lib.rs:284-287)
            be.upload_state(pos, vel)
            be.forces_resident()
            e_pot, e_kin = be.resident_energies()
            dcd.write_frame(pos[0].astype(np.float32), pos[1].astype(np.float32), pos[2].astype(np.float32))
            csv.write_row(first_step, first_step * dt_ps, e_pot, e_kin)
            done = 0
            while done < n_steps:
                # whole frame intervals per batch, so the ring never overflows
                chunk = min(n_steps - done, frames_per_batch * frame_interval)
                be.run_resident(dt_ps, chunk, first_step=first_step + done)
                done += chunk
                fr = be.frames_take()
                dcd.write_frames(fr["xyz"])
                for s, ep, ek in zip(fr["step"], fr["e_pot"], fr["e_kin"]):
                    csv.write_row(int(s), int(s) * dt_ps, float(ep), float(ek))
            be.download_state(pos, vel)
            return dcd.n_frames
    finally:
        be.frames_enable(0, 0)
