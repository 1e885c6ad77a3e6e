"""`geodesic run config.toml` on the CUDA backend: the run loop of
geodesic/src/lib.rs:175-345 with every step on the device.

Single system (the reference's `[system]` table), the order of lib.rs:187-333:
parse the prmtop and inpcrd (paths resolved against the config file's
directory, lib.rs:63-66), promote H bonds to constraints when
`constrain_hydrogens`, project the initial velocities onto the constraint
tangent space (lib.rs:270-282), evaluate the forces, write frame 0 (f32
positions, potential and kinetic energy), then `n_steps` BAB + RATTLE steps
with a frame every `frame_interval` steps: DCD frame, CSV row and the energy
drift check of `[monitoring]` (lib.rs:363-386: |E - E0| above the threshold
warns on stderr or stops with `EnergyDriftError` after that frame is written).
The device records the frames itself and the host drains them
`frames_per_batch` at a time, so the steps between frames never wait for the
host.

Batch (a `[[system]]` array): the systems run in one device context
(gm_create_ensemble), each with its own DCD and CSV (the `{system}` output
paths).  The device advances all systems frame interval by frame interval;
after each interval the host reads the per-system energies and positions and
writes every system's frame, CSV row and drift check.  Each file holds what
the system's own single run writes (with constraints, the batch's SHAKE and
RATTLE iterate every cluster to the batch's largest count, each converged to
the tolerance).

`RunSummary` mirrors lib.rs:49-57: `final_potential` is the potential of the
last force evaluation and `final_kinetic` the kinetic energy of the last
frame, as the reference keeps them.
"""
from __future__ import annotations

import dataclasses
import os
import sys

import numpy as np

from . import amber
from .backend import CudaBackend, NumericalError
from .config import Backend, Config, ConfigError, DriftAction, rust_f64
from .trajectory import DcdWriter, EnergyLogWriter


_INT32_MAX = 2**31 - 1


class SimIoError(OSError):
    """IoError (geodesic-core/src/error.rs:26-32): a file that could not be read."""

    def __init__(self, path, source: OSError):
        super().__init__(f"I/O error at '{path}': {source}")
        self.path, self.source = path, source


class EnergyDriftError(NumericalError):
    """NumericalError::EnergyDrift (error.rs:41-47), raised by `[monitoring]`
    with energy_drift_action = "stop"."""

    def __init__(self, step: int, drift_kcal: float, threshold_kcal: float, system: str | None = None):
        msg = (f"energy drift {rust_f64(drift_kcal)} kcal/mol exceeds threshold {rust_f64(threshold_kcal)} kcal/mol "
               f"at step {step}")
        RuntimeError.__init__(self, msg if system is None else f"system {system}: {msg}")
        self.status = None
        self.step, self.drift_kcal, self.threshold_kcal, self.system = step, drift_kcal, threshold_kcal, system


@dataclasses.dataclass
class RunSummary:
    """RunSummary (lib.rs:49-57); `name` is the system's name in a batch."""

    n_steps: int
    n_frames: int
    final_potential: float
    final_kinetic: float
    trajectory: str
    energy_log: str
    name: str | None = None


def _read(path) -> str:
    try:
        with open(path, encoding="utf-8") as f:
            return f.read()
    except OSError as e:
        raise SimIoError(path, e) from None


def _resolve(base: str, path: str) -> str:
    """lib.rs:63-66: relative to the config file's directory; an absolute path
    stays as it is."""
    return os.path.join(base, path)


def _load_system(config: Config, base: str, k: int):
    s = config.systems[k]
    atoms, topo = amber.parse_prmtop(_read(_resolve(base, s.prmtop)))
    state = amber.parse_inpcrd(_read(_resolve(base, s.inpcrd)), atoms.n, False)
    if config.constrain_hydrogens:
        topo = amber.promote_hydrogen_bonds(topo, atoms)
    return atoms, topo, state


def _cuda_backend(atoms_list, topo_list, params):
    if len(atoms_list) == 1:
        return CudaBackend(atoms_list[0], topo_list[0], params)
    return CudaBackend.ensemble(atoms_list, topo_list, params)


class _DriftMonitor:
    """check_energy_drift (lib.rs:363-386) against the frame-0 energy."""

    def __init__(self, config: Config, e0: float, system: str | None = None):
        self.m, self.e0, self.system = config.monitoring, e0, system

    def __call__(self, step: int, e_pot: float, e_kin: float) -> None:
        if self.m is None:
            return
        drift = abs((e_pot + e_kin) - self.e0)
        if drift <= self.m.energy_drift_threshold_kcal:
            return
        if self.m.energy_drift_action is DriftAction.WARN:
            where = "" if self.system is None else f" in system {self.system}"
            print(f"warning: energy drift {drift:.4f} kcal/mol exceeds threshold "
                  f"{self.m.energy_drift_threshold_kcal:.4f} at step {step}{where}", file=sys.stderr)
            return
        raise EnergyDriftError(step, drift, self.m.energy_drift_threshold_kcal, self.system)


def run_from_config_file(config_path, make_backend=None):
    """`run_from_config_file` (lib.rs:175-180): a RunSummary for a `[system]`
    config, a list of them (one per system, in order) for a `[[system]]`
    batch.  `make_backend(atoms_list, topo_list, params)` builds the backend
    (default: `CudaBackend`, or its batch form for several systems)."""
    config_path = os.fspath(config_path)
    config = Config.from_toml_str(_read(config_path))
    return run(config, os.path.dirname(config_path), make_backend)


def run(config: Config, base: str = "", make_backend=None):
    """`run` (lib.rs:187-345) for `backend = "cuda"`."""
    if config.backend is not Backend.CUDA:
        raise ConfigError.invalid_value("run.backend", config.backend.value,
                                        'this package runs the "cuda" backend; "cpu", "gpu" and "hybrid" are the '
                                        "reference binary's")
    if config.frame_interval == 0:
        # the reference's loop takes step % frame_interval; zero is not a period
        raise ConfigError.invalid_value("run.frame_interval", "0", "must be greater than zero")
    if config.frame_interval > _INT32_MAX:
        raise ConfigError.invalid_value("run.frame_interval", str(config.frame_interval),
                                        "the device records frames at intervals below 2^31 steps")
    make_backend = make_backend or _cuda_backend
    loaded = [_load_system(config, base, k) for k in range(len(config.systems))]
    atoms_list = [a for a, _, _ in loaded]
    topo_list = [t for _, t, _ in loaded]
    pos = np.ascontiguousarray(np.concatenate([s.pos for _, _, s in loaded], axis=1), dtype=np.float64)
    vel = np.ascontiguousarray(np.concatenate([s.vel for _, _, s in loaded], axis=1), dtype=np.float64)
    paths = [tuple(_resolve(base, p) for p in config.outputs(k)) for k in range(len(config.systems))]
    be = make_backend(atoms_list, topo_list, config.sim_params())
    try:
        if not config.batch:
            return _run_single(config, be, pos, vel, paths[0])
        return _run_batch(config, be, pos, vel, paths, [a.n for a in atoms_list])
    finally:
        be.close()


def _initial_state(config: Config, be, pos, vel):
    """lib.rs:261-282: the first list build (which wraps a periodic system
    into the box, neighbor.rs:10-16), the velocity projection on those
    positions, then the resident state's forces and energies.  The first
    build is the backend's own list build on the host arrays, so the wrap
    runs once, on the device, as the reference runs it once; frame 0 and the
    projection see the wrapped positions, and the resident forces use the
    list that build made (the uploaded positions are its own, so nothing is
    wrapped twice)."""
    be.build_neighbor_list(pos)
    be.constrain_velocities(pos, vel, 0)
    be.upload_state(pos, vel)
    be.forces_resident()


def _run_single(config: Config, be, pos, vel, paths) -> RunSummary:
    n, fi, dt = pos.shape[1], config.frame_interval, config.dt
    traj, log = paths
    be.frames_enable(fi, config.frames_per_batch)
    with DcdWriter(traj, n, fi, dt) as dcd, EnergyLogWriter(log, n) as csv:
        _initial_state(config, be, pos, vel)
        e_pot, e_kin = be.resident_energies()
        dcd.write_frame(pos[0].astype(np.float32), pos[1].astype(np.float32), pos[2].astype(np.float32))
        csv.write_row(0, 0.0, e_pot, e_kin)
        monitor = _DriftMonitor(config, e_pot + e_kin)
        last_kin = e_kin
        done = 0
        while done < config.n_steps:
            # whole frame intervals per batch, so the ring never overflows
            chunk = min(config.n_steps - done, config.frames_per_batch * fi)
            be.run_resident(dt, chunk, first_step=done)
            done += chunk
            fr = be.frames_take()
            for k in range(len(fr["step"])):
                step = int(fr["step"][k])
                ep, ek = float(fr["e_pot"][k]), float(fr["e_kin"][k])
                xyz = fr["xyz"][k]
                dcd.write_frame(xyz[0], xyz[1], xyz[2])
                csv.write_row(step, step * dt, ep, ek)
                last_kin = ek
                monitor(step, ep, ek)
        be.download_state(pos, vel)
        final_pot, _ = be.resident_energies()
        return RunSummary(config.n_steps, dcd.n_frames, final_pot, last_kin, traj, log)


def _ensure_open_files(n: int) -> None:
    """Raises the soft limit on open files to hold n (two per system of a
    batch), up to the hard limit."""
    try:
        import resource
    except ImportError:
        return
    soft, hard = resource.getrlimit(resource.RLIMIT_NOFILE)
    if soft != resource.RLIM_INFINITY and soft < n:
        want = n if hard == resource.RLIM_INFINITY else min(n, hard)
        resource.setrlimit(resource.RLIMIT_NOFILE, (want, hard))


def _run_batch(config: Config, be, pos, vel, paths, sizes) -> list:
    fi, dt = config.frame_interval, config.dt
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    ns = len(sizes)
    _ensure_open_files(2 * ns + 64)
    dcds, csvs = [], []
    try:
        for k in range(ns):
            dcds.append(DcdWriter(paths[k][0], sizes[k], fi, dt))
            csvs.append(EnergyLogWriter(paths[k][1], sizes[k]))
        _initial_state(config, be, pos, vel)
        ep, ek = be.ensemble_energies()
        monitors = [_DriftMonitor(config, ep[k] + ek[k], config.systems[k].name) for k in range(ns)]
        last_kin = np.array(ek, dtype=np.float64)

        def write_frames(step, ep, ek, check):
            p32 = pos.astype(np.float32)
            for k in range(ns):
                a, b = off[k], off[k + 1]
                dcds[k].write_frame(p32[0, a:b], p32[1, a:b], p32[2, a:b])
                csvs[k].write_row(step, step * dt, float(ep[k]), float(ek[k]))
            last_kin[:] = ek
            if check:
                for k in range(ns):
                    monitors[k](step, float(ep[k]), float(ek[k]))

        write_frames(0, ep, ek, False)
        done = 0
        while done < config.n_steps:
            nxt = min(config.n_steps, (done // fi + 1) * fi)
            be.run_resident(dt, nxt - done, first_step=done)
            done = nxt
            if done % fi == 0:
                ep, ek = be.ensemble_energies()
                be.download_state(pos, vel)
                write_frames(done, ep, ek, True)
        ep, _ = be.ensemble_energies()
        out = []
        for k in range(ns):
            out.append(RunSummary(config.n_steps, dcds[k].n_frames, float(ep[k]), float(last_kin[k]), paths[k][0],
                                  paths[k][1], config.systems[k].name))
        return out
    finally:
        for w in dcds + csvs:
            w.close()


def main(argv=None) -> int:
    """`geodesic run <config.toml>` (geodesic/src/main.rs) for this backend."""
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("usage: python -m geodesic_cuda.run <config.toml>", file=sys.stderr)
        return 2
    res = run_from_config_file(argv[0])
    for s in res if isinstance(res, list) else [res]:
        tag = f"{s.name}: " if s.name is not None else ""
        print(f"{tag}{s.n_steps} steps, {s.n_frames} frames, E_pot {s.final_potential:.3f} kcal/mol, "
              f"E_kin {s.final_kinetic:.3f} kcal/mol -> {s.trajectory}, {s.energy_log}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
