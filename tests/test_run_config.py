"""`config.toml` and the run loop (CPU only).

Config: the reference's schema, defaults, error kinds and messages
(geodesic-io/src/config.rs:1-265, geodesic-core/src/error.rs:65-79), on the
config of geodesic/tests/golden_reference.rs:39-71 and on broken variants of
it; then the additions (`backend = "cuda"`, `[cuda]`, `[[system]]` batches).

Run loop: `geodesic_cuda.run` driven through an oracle-backed stand-in of the
backend's resident methods (tests/oracle_resident.py) writes the DCD frames
and CSV rows that `oracle.run` (the restatement of lib.rs:187-333) gives for
the same files: the initial velocity projection, frame 0, frames drained in
batches across frame intervals, a step count that is not a multiple of the
frame interval, per-system files of a batch, and the energy drift monitor's
warn and stop."""
import os
import sys

import numpy as np
import pytest

from geodesic_cuda import amber, config, run, synth, trajectory
from geodesic_cuda.config import ConfigError

import amber_files
import oracle
import oracle_resident

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_fixtures import read_dcd  # noqa: E402

GOLDEN_CONFIG = """
[run]
n_steps        = 99
frame_interval = 1
backend        = "cpu"
n_threads      = 1

[system]
prmtop   = "ala_dipeptide.prmtop"
inpcrd   = "ala_dipeptide.inpcrd"
box_size = [1000.0, 1000.0, 1000.0]
periodic = false

[integrator]
dt           = 0.001
total_energy = 5.12

[nonbonded]
r_cutoff = 12.0
r_skin   = 14.0
r_switch = 10.0

[constraints]
max_iter  = 100
tolerance = 1.0e-8

[output]
trajectory = "out.dcd"
energy_log = "out.csv"
"""


def edit(text, old, new):
    assert old in text, old
    return text.replace(old, new, 1)


def parse_error(text) -> ConfigError:
    with pytest.raises(ConfigError) as e:
        config.Config.from_toml_str(text)
    return e.value


# ------------------------------------------------------------ config.rs

def test_reference_golden_config_parses():
    c = config.Config.from_toml_str(GOLDEN_CONFIG)
    assert (c.n_steps, c.frame_interval, c.backend, c.n_threads) == (99, 1, config.Backend.CPU, 1)
    assert (c.prmtop, c.inpcrd, c.box_size, c.periodic) == ("ala_dipeptide.prmtop", "ala_dipeptide.inpcrd",
                                                            (1000.0,) * 3, False)
    assert (c.dt, c.total_energy, c.r_cutoff, c.r_skin, c.r_switch) == (0.001, 5.12, 12.0, 14.0, 10.0)
    assert (c.max_constr_iter, c.constr_tol) == (100, 1e-8)
    assert c.constrain_hydrogens is True  # config.rs:54-61 default
    assert c.monitoring is None and c.batch is False
    assert (c.trajectory, c.energy_log) == ("out.dcd", "out.csv")
    assert (c.precision, c.frames_per_batch) == ("mixed", 64)
    for b in ("gpu", "hybrid", "cuda"):
        assert config.Config.from_toml_str(edit(GOLDEN_CONFIG, '"cpu"', f'"{b}"')).backend.value == b
    p = config.Config.from_toml_str(edit(GOLDEN_CONFIG, '"cpu"', '"cuda"')).sim_params()
    assert (p.box_size, p.r_cutoff, p.r_skin, p.r_switch, p.max_constr_iter, p.constr_tol) == (
        (1000.0,) * 3, 12.0, 14.0, 10.0, 100, 1e-8)


def test_integers_are_accepted_for_reals_and_optional_tables_read():
    text = edit(GOLDEN_CONFIG, "dt           = 0.001", "dt           = 1")
    text += '\n[monitoring]\nenergy_drift_threshold_kcal = 2\nenergy_drift_action = "stop"\n'
    c = config.Config.from_toml_str(text)
    assert c.dt == 1.0 and isinstance(c.dt, float)
    assert c.monitoring == config.MonitoringConfig(2.0, config.DriftAction.STOP)
    c = config.Config.from_toml_str(GOLDEN_CONFIG + '\n[cuda]\nprecision = "fp64"\nframes_per_batch = 8\n'
                                    'bonded_min_image = true\n')
    assert (c.precision, c.frames_per_batch, c.bonded_min_image) == ("fp64", 8, True)
    assert c.sim_params().bonded_min_image is True
    assert config.Config.from_toml_str(GOLDEN_CONFIG).sim_params().bonded_min_image is False


@pytest.mark.parametrize("old,new,key", [
    ("n_threads      = 1", "n_threads      = 1\nthreads = 2", "threads"),
    ("periodic = false", "periodic = false\nwrap = true", "wrap"),
    ("tolerance = 1.0e-8", "tolerance = 1.0e-8\nshake = 1", "shake"),
    ("[output]", "[extra]\nx = 1\n\n[output]", "extra"),
    ("periodic = false", 'periodic = false\nname = "a"', "name"),  # `name` belongs to the batch form only
])
def test_unknown_keys(old, new, key):
    e = parse_error(edit(GOLDEN_CONFIG, old, new))
    assert e.kind == "UnknownKey" and str(e) == f"unknown config key: {key}"


@pytest.mark.parametrize("old,key", [
    ("n_steps        = 99\n", "n_steps"),
    ("box_size = [1000.0, 1000.0, 1000.0]\n", "box_size"),
    ("total_energy = 5.12\n", "total_energy"),
    ("energy_log = \"out.csv\"\n", "energy_log"),
    ("[nonbonded]\nr_cutoff = 12.0\nr_skin   = 14.0\nr_switch = 10.0\n", "nonbonded"),
])
def test_missing_keys(old, key):
    e = parse_error(edit(GOLDEN_CONFIG, old, ""))
    assert e.kind == "MissingRequired" and str(e) == f"missing required config key: {key}"


def test_bad_backend_and_drift_action():
    e = parse_error(edit(GOLDEN_CONFIG, '"cpu"', '"metal"'))
    assert e.kind == "InvalidValue" and str(e) == (
        "invalid value for key 'run.backend': 'metal' (expected \"cpu\", \"gpu\", \"hybrid\", or \"cuda\")")
    e = parse_error(GOLDEN_CONFIG + '\n[monitoring]\nenergy_drift_threshold_kcal = 1.0\nenergy_drift_action = "halt"\n')
    assert str(e) == "invalid value for key 'monitoring.energy_drift_action': 'halt' (expected \"warn\" or \"stop\")"


@pytest.mark.parametrize("old,new", [
    ("n_steps        = 99", "n_steps        = -1"),
    ("n_steps        = 99", "n_steps        = 99.0"),
    ("frame_interval = 1", "frame_interval = 4294967296"),
    ("backend        = \"cpu\"", "backend        = 3"),
    ("box_size = [1000.0, 1000.0, 1000.0]", "box_size = [1000.0, 1000.0]"),
    ("periodic = false", "periodic = 0"),
    ("dt           = 0.001", "dt           = \"0.001\""),
    ("max_iter  = 100", "max_iter  = true"),
    ("[run]", "[run"),  # TOML syntax
])
def test_type_and_syntax_errors_are_invalid_values_of_the_file(old, new):
    e = parse_error(edit(GOLDEN_CONFIG, old, new))
    assert e.kind == "InvalidValue" and e.key == "config.toml"


@pytest.mark.parametrize("old,new,message", [
    ("n_steps        = 99", "n_steps        = 0", "run.n_steps must be greater than zero"),
    ("box_size = [1000.0, 1000.0, 1000.0]", "box_size = [1000.0, 0.0, 1000.0]",
     "system.box_size components must be positive"),
    ("dt           = 0.001", "dt           = -0.001", "integrator.dt must be positive"),
    ("r_switch = 10.0", "r_switch = 12.0",
     "nonbonded radii must satisfy r_switch < r_cutoff < r_skin (got r_switch=12, r_cutoff=12, r_skin=14)"),
    ("r_skin   = 14.0", "r_skin   = 11.5",
     "nonbonded radii must satisfy r_switch < r_cutoff < r_skin (got r_switch=10, r_cutoff=12, r_skin=11.5)"),
    ("max_iter  = 100", "max_iter  = 0", "constraints.max_iter must be greater than zero"),
    ("tolerance = 1.0e-8", "tolerance = 0.0", "constraints.tolerance must be positive"),
])
def test_physically_invalid(old, new, message):
    e = parse_error(edit(GOLDEN_CONFIG, old, new))
    assert e.kind == "PhysicallyInvalid" and str(e) == f"physically invalid configuration: {message}"


def test_validation_order_follows_the_reference():
    # n_steps is checked before dt, dt before the radii
    text = edit(edit(GOLDEN_CONFIG, "n_steps        = 99", "n_steps        = 0"), "dt           = 0.001",
                "dt           = 0.0")
    assert "n_steps" in str(parse_error(text))
    text = edit(edit(GOLDEN_CONFIG, "dt           = 0.001", "dt           = 0.0"), "r_switch = 10.0",
                "r_switch = 20.0")
    assert "integrator.dt" in str(parse_error(text))


@pytest.mark.parametrize("x,s", [(12.0, "12"), (0.1, "0.1"), (11.5, "11.5"), (1e-05, "0.00001"),
                                 (1.5e20, "150000000000000000000"), (1e16, "10000000000000000"),
                                 (123456789.125, "123456789.125"), (-0.0, "-0"), (float("nan"), "NaN"),
                                 (float("inf"), "inf"), (2.5e-7, "0.00000025"), (-3.0, "-3")])
def test_rust_float_display(x, s):
    assert config.rust_f64(x) == s


BATCH_SYSTEMS = """
[[system]]
name     = "alpha"
prmtop   = "a.prmtop"
inpcrd   = "a.inpcrd"
box_size = [1000.0, 1000.0, 1000.0]

[[system]]
prmtop   = "b.prmtop"
inpcrd   = "b.inpcrd"
box_size = [1000.0, 1000.0, 1000.0]
"""


def batch_config(systems=BATCH_SYSTEMS, traj="traj_{system}.dcd", log="energy_{system}.csv"):
    text = edit(GOLDEN_CONFIG, """[system]
prmtop   = "ala_dipeptide.prmtop"
inpcrd   = "ala_dipeptide.inpcrd"
box_size = [1000.0, 1000.0, 1000.0]
periodic = false
""", systems)
    text = edit(text, 'trajectory = "out.dcd"', f'trajectory = "{traj}"')
    return edit(text, 'energy_log = "out.csv"', f'energy_log = "{log}"')


def test_batch_form():
    c = config.Config.from_toml_str(batch_config())
    assert c.batch and [s.name for s in c.systems] == ["alpha", "1"]
    assert [s.prmtop for s in c.systems] == ["a.prmtop", "b.prmtop"]
    assert c.outputs(0) == ("traj_alpha.dcd", "energy_alpha.csv")
    assert c.outputs(1) == ("traj_1.dcd", "energy_1.csv")
    one = config.Config.from_toml_str(batch_config(BATCH_SYSTEMS.split("[[system]]", 2)[1].join(["[[system]]", ""]),
                                                   traj="t.dcd", log="e.csv"))
    assert one.batch and len(one.systems) == 1 and one.outputs(0) == ("t.dcd", "e.csv")


@pytest.mark.parametrize("systems,traj,key", [
    (BATCH_SYSTEMS, "traj.dcd", "output.trajectory"),
    (BATCH_SYSTEMS.replace('name     = "alpha"', 'name     = "1"'), "traj_{system}.dcd", "system.name"),
    (BATCH_SYSTEMS.replace('name     = "alpha"', 'name     = ""'), "traj_{system}.dcd", "system.name"),
    (BATCH_SYSTEMS.replace("box_size = [1000.0, 1000.0, 1000.0]\n", "box_size = [900.0, 1000.0, 1000.0]\n", 1),
     "traj_{system}.dcd", "system.box_size"),
    (BATCH_SYSTEMS + "periodic = true\n", "traj_{system}.dcd", "system.box_size"),
    (None, "traj_{system}.dcd", "system"),
])
def test_batch_errors(systems, traj, key):
    # None: an empty array, `system = []` at the top of the file
    text = batch_config(systems, traj=traj) if systems is not None else "system = []\n" + batch_config("", traj=traj)
    e = parse_error(text)
    assert e.kind == "InvalidValue" and e.key == key, str(e)


def test_cuda_table_errors():
    e = parse_error(GOLDEN_CONFIG + '\n[cuda]\nprecision = "fp16"\n')
    assert e.key == "cuda.precision"
    for bad in (0, 2**31):
        e = parse_error(GOLDEN_CONFIG + f"\n[cuda]\nframes_per_batch = {bad}\n")
        assert e.key == "cuda.frames_per_batch"
    e = parse_error(GOLDEN_CONFIG + "\n[cuda]\ngraphs = true\n")
    assert e.kind == "UnknownKey"


# ------------------------------------------------------------ run loop

def write_case(tmp_path, systems, n_steps, frame_interval, constrain=True, frames_per_batch=3, extra="", tol=1e-8,
               files=None, box=1000.0, periodic=False, centre=None, min_image=False):
    """Writes each (name, n_atoms, seed, h_fraction) system's AMBER files and
    a config running them; returns the config path.  `files`: (name, prmtop,
    inpcrd) entries already in tmp_path, used instead.  `centre`: where the
    system's centroid is put (default: where the generator put it)."""
    entries = list(files or [])
    for name, n, seed, hf in ([] if files else systems):
        atoms, topo, state, _ = synth.generate(n, seed=seed, h_fraction=hf, temperature=300.0, relax_iters=200)
        if centre is not None:
            state.pos = state.pos - state.pos.mean(axis=1, keepdims=True) + np.asarray(centre, float)[:, None]
        prm, crd = amber_files.write_system(tmp_path, name, atoms, topo, state)
        entries.append((name, prm, crd))
    batch = len(entries) > 1
    box_text = f"box_size = [{box!r}, {box!r}, {box!r}]\nperiodic = {'true' if periodic else 'false'}\n"
    if batch:
        sys_text = "".join(f'[[system]]\nname = "{nm}"\nprmtop = "{p}"\ninpcrd = "{c}"\n{box_text}\n'
                           for nm, p, c in entries)
        traj, log = "traj_{system}.dcd", "energy_{system}.csv"
    else:
        nm, p, c = entries[0]
        sys_text = f'[system]\nprmtop = "{p}"\ninpcrd = "{c}"\n{box_text}\n'
        traj, log = "traj.dcd", "energy.csv"
    text = f"""[run]
n_steps = {n_steps}
frame_interval = {frame_interval}
backend = "cuda"
n_threads = 1

{sys_text}[integrator]
dt = 0.002
total_energy = 0.0

[nonbonded]
r_cutoff = 10.0
r_skin = 11.0
r_switch = 8.0

[constraints]
max_iter = 100
tolerance = {tol!r}
constrain_hydrogens = {"true" if constrain else "false"}

[output]
trajectory = "{traj}"
energy_log = "{log}"

[cuda]
frames_per_batch = {frames_per_batch}
bonded_min_image = {"true" if min_image else "false"}
{extra}"""
    path = tmp_path / "config.toml"
    path.write_text(text)
    return path


def oracle_expected(tmp_path, stem, n_steps, frame_interval, constrain=True, tol=1e-8, box=1000.0, periodic=False,
                    min_image=False):
    atoms, topo, state = amber.load(str(tmp_path / f"{stem}.prmtop"), str(tmp_path / f"{stem}.inpcrd"))
    if constrain:
        topo = amber.promote_hydrogen_bonds(topo, atoms)
    p = oracle.make_params(box=(box,) * 3, periodic=periodic, r_cutoff=10.0, r_skin=11.0, r_switch=8.0,
                           max_constr_iter=100, constr_tol=tol, n_threads=1, bonded_min_image=min_image)
    frames, pot, kin = oracle.run(atoms, topo, p, np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel),
                                  0.002, n_steps, frame_interval)
    return atoms.n, frames, pot, kin


def expected_csv(tmp_path, n_atoms, frame_interval, pot, kin):
    path = tmp_path / "expected.csv"
    with trajectory.EnergyLogWriter(path, n_atoms) as w:
        for k in range(len(pot)):
            step = k * frame_interval
            w.write_row(step, step * 0.002, pot[k], kin[k])
    return path.read_text()


@pytest.mark.parametrize("n_steps,constrain", [(40, True), (23, False)])
def test_single_run_writes_the_oracle_run(tmp_path, n_steps, constrain):
    cfg = write_case(tmp_path, [("sys", 300, 41, 0.3)], n_steps, 5, constrain=constrain)
    cwd = os.getcwd()
    os.chdir(tmp_path.parent)  # paths resolve against the config's directory, not the working directory
    try:
        summary = run.run_from_config_file(os.path.join(tmp_path.name, "config.toml"), make_backend=oracle_resident.make)
    finally:
        os.chdir(cwd)
    n, frames, pot, kin = oracle_expected(tmp_path, "sys", n_steps, 5, constrain)
    header, dcd = read_dcd(tmp_path / "traj.dcd")
    assert header["nset"] == len(frames) == n_steps // 5 + 1 and header["natom"] == n and header["nsavc"] == 5
    assert np.array_equal(dcd.view(np.uint32), frames.view(np.uint32))
    assert (tmp_path / "energy.csv").read_text() == expected_csv(tmp_path, n, 5, pot, kin)
    assert summary.n_frames == len(frames) and summary.n_steps == n_steps
    assert summary.final_kinetic == kin[-1]
    if n_steps % 5 == 0:
        assert summary.final_potential == pot[-1]
    assert summary.trajectory == os.path.join(tmp_path.name, "traj.dcd")


def test_projection_comes_first_and_frames_drain_in_batches(tmp_path):
    cfg = write_case(tmp_path, [("sys", 200, 43, 0.3)], 40, 5, frames_per_batch=3)
    made = []

    def make(*a):
        made.append(oracle_resident.make(*a))
        return made[-1]

    run.run_from_config_file(cfg, make_backend=make)
    be = made[0]
    assert be.calls[:5] == [("frames_enable", 5, 3), "build_neighbor_list", "constrain_velocities", "upload_state",
                            "forces_resident"]
    runs = [c for c in be.calls if isinstance(c, tuple) and c[0] == "run_resident"]
    assert runs == [("run_resident", 15, 0), ("run_resident", 15, 15), ("run_resident", 10, 30)]
    assert be.closed


def test_batch_run_writes_each_systems_own_run(tmp_path):
    systems = [("a", 260, 44, 0.3), ("b", 190, 45, 0.0), ("c", 330, 46, 0.25)]
    cfg = write_case(tmp_path, systems, 30, 10)
    summaries = run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    assert [s.name for s in summaries] == ["a", "b", "c"]
    for (name, _, _, _), s in zip(systems, summaries):
        n, frames, pot, kin = oracle_expected(tmp_path, name, 30, 10)
        header, dcd = read_dcd(tmp_path / f"traj_{name}.dcd")
        assert header["nset"] == 4 and header["natom"] == n
        assert np.array_equal(dcd.view(np.uint32), frames.view(np.uint32)), name
        assert (tmp_path / f"energy_{name}.csv").read_text() == expected_csv(tmp_path, n, 10, pot, kin), name
        assert (s.n_frames, s.final_potential, s.final_kinetic) == (4, pot[-1], kin[-1])
        assert s.trajectory == str(tmp_path / f"traj_{name}.dcd")


def test_drift_stop_raises_after_writing_the_frame(tmp_path):
    extra = '\n[monitoring]\nenergy_drift_threshold_kcal = 0.0\nenergy_drift_action = "stop"\n'
    cfg = write_case(tmp_path, [("sys", 200, 47, 0.0)], 40, 5, constrain=False, extra=extra)
    with pytest.raises(run.EnergyDriftError) as e:
        run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    assert e.value.step == 5 and e.value.threshold_kcal == 0.0
    assert str(e.value).startswith("energy drift ") and str(e.value).endswith(
        " kcal/mol exceeds threshold 0 kcal/mol at step 5")
    n, frames, pot, kin = oracle_expected(tmp_path, "sys", 5, 5, constrain=False)
    header, dcd = read_dcd(tmp_path / "traj.dcd")
    assert header["nset"] == 2 and np.array_equal(dcd, frames)  # frames 0 and 5, count patched on close
    assert len((tmp_path / "energy.csv").read_text().splitlines()) == 3
    assert e.value.drift_kcal == abs((pot[1] + kin[1]) - (pot[0] + kin[0]))  # |E - E0|, lib.rs:367-368


def test_drift_warn_keeps_running(tmp_path, capsys):
    extra = '\n[monitoring]\nenergy_drift_threshold_kcal = 0.0\nenergy_drift_action = "warn"\n'
    cfg = write_case(tmp_path, [("a", 150, 48, 0.0), ("b", 170, 49, 0.0)], 20, 10, constrain=False, extra=extra)
    out = run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    assert [s.n_frames for s in out] == [3, 3]
    err = capsys.readouterr().err.splitlines()
    assert len(err) == 4 and all(line.startswith("warning: energy drift ") for line in err)
    assert err[0].endswith(" kcal/mol exceeds threshold 0.0000 at step 10 in system a")


def test_run_errors(tmp_path):
    cfg = write_case(tmp_path, [("sys", 100, 50, 0.0)], 10, 5)
    text = cfg.read_text()
    cfg.write_text(edit(text, 'backend = "cuda"', 'backend = "cpu"'))
    with pytest.raises(ConfigError) as e:
        run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    assert e.value.key == "run.backend"
    cfg.write_text(edit(text, "frame_interval = 5", "frame_interval = 0"))
    with pytest.raises(ConfigError) as e:
        run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    assert e.value.key == "run.frame_interval"
    cfg.write_text(edit(text, "frame_interval = 5", "frame_interval = 2147483648"))
    with pytest.raises(ConfigError) as e:
        run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    assert e.value.key == "run.frame_interval"
    cfg.write_text(edit(text, 'prmtop = "sys.prmtop"', 'prmtop = "missing.prmtop"'))
    with pytest.raises(run.SimIoError) as e:
        run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    assert str(e.value).startswith(f"I/O error at '{tmp_path / 'missing.prmtop'}': ")
    with pytest.raises(run.SimIoError):
        run.run_from_config_file(tmp_path / "no_such.toml", make_backend=oracle_resident.make)


@pytest.mark.parametrize("centre,min_image", [((95.0, -25.0, 155.0), False), ((0.0, 0.0, 0.0), True)])
def test_periodic_run_wraps_before_frame_zero(tmp_path, centre, min_image):
    """A periodic system placed outside the box (moved inside whole by the
    first wrap) or around a corner (split by it; with bonded_min_image): the
    wrap comes before frame 0 and the velocity projection, as in the
    reference's first list build (lib.rs:261-282), so the files are those of
    oracle.run, bit for bit."""
    cfg = write_case(tmp_path, [("sys", 250, 52, 0.3)], 20, 5, box=60.0, periodic=True, centre=centre,
                     min_image=min_image)
    run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    n, frames, pot, kin = oracle_expected(tmp_path, "sys", 20, 5, box=60.0, periodic=True, min_image=min_image)
    header, dcd = read_dcd(tmp_path / "traj.dcd")
    assert np.array_equal(dcd.view(np.uint32), frames.view(np.uint32))
    assert np.all((dcd[0] >= 0.0) & (dcd[0] < 60.0))  # frame 0 is already in the box
    assert (tmp_path / "energy.csv").read_text() == expected_csv(tmp_path, n, 5, pot, kin)


def test_periodic_run_wraps_once():
    """A coordinate just below 0 (-1e-17) wraps to exactly the box length L
    (L - 1e-17 rounds to L); a second wrap would turn it into 0.  The run's
    initial state wraps once, as the reference's first list build does
    (lib.rs:261-282, neighbor.rs:10-16): the positions for frame 0 and the
    projection hold L, and the resident state keeps them.  (An inpcrd file
    cannot hold such a value, its fields have 7 decimals, so the state is
    given directly.)"""
    atoms, topo, state, _ = synth.generate(250, seed=55, h_fraction=0.3, temperature=300.0, relax_iters=200)
    pos = state.pos - state.pos.mean(axis=1, keepdims=True) + 30.0
    k = int(np.argmin(pos[0]))
    pos[0, k] = -1e-17
    pos = np.ascontiguousarray(pos)
    vel = np.ascontiguousarray(state.vel.copy())
    params = backend_params(box_size=(60.0,) * 3, periodic=True)
    be = oracle_resident.make([atoms], [topo], params)
    run._initial_state(None, be, pos, vel)
    assert pos[0, k] == 60.0
    ref = np.ascontiguousarray(state.pos - state.pos.mean(axis=1, keepdims=True) + 30.0)
    ref[0, k] = -1e-17
    oracle.CpuBackend(atoms, topo, be.p).build_neighbor_list(ref)
    assert np.array_equal(pos, ref)
    p2, v2 = np.zeros_like(pos), np.zeros_like(vel)
    be.download_state(p2, v2)
    assert np.array_equal(p2, ref)


def backend_params(**kw):
    from geodesic_cuda import backend
    base = dict(r_cutoff=10.0, r_skin=11.0, r_switch=8.0, max_constr_iter=100, constr_tol=1e-8)
    base.update(kw)
    return backend.SimParams(**base)


def test_periodic_batch_wraps_every_system(tmp_path):
    """A periodic [[system]] batch (one shared box, bonded_min_image): each
    system placed around a corner of the box writes oracle.run's files."""
    systems = [("a", 200, 53, 0.3), ("b", 260, 54, 0.2)]
    cfg = write_case(tmp_path, systems, 20, 10, box=60.0, periodic=True, centre=(0.0, 60.0, -3.0), min_image=True)
    out = run.run_from_config_file(cfg, make_backend=oracle_resident.make)
    for (name, _, _, _), s in zip(systems, out):
        n, frames, pot, kin = oracle_expected(tmp_path, name, 20, 10, box=60.0, periodic=True, min_image=True)
        header, dcd = read_dcd(tmp_path / f"traj_{name}.dcd")
        assert np.array_equal(dcd.view(np.uint32), frames.view(np.uint32)), name
        assert (tmp_path / f"energy_{name}.csv").read_text() == expected_csv(tmp_path, n, 10, pot, kin), name
