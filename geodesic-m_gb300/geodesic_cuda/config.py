"""`config.toml` for the CUDA backend: the reference's schema, defaults,
validation and error messages (geodesic-io/src/config.rs:1-265), read with
Python's `tomllib`, plus `backend = "cuda"` and a batch form.

Schema (every table rejects unknown keys, like the reference's
`#[serde(deny_unknown_fields)]`, config.rs:5-80):

  [run]          n_steps (u64), frame_interval (u32), backend (string), n_threads (usize)
  [system]       prmtop, inpcrd (paths), box_size ([f64; 3]), periodic (bool, default false)
  [integrator]   dt, total_energy (f64)
  [nonbonded]    r_cutoff, r_skin, r_switch (f64)
  [constraints]  max_iter (u32), tolerance (f64), constrain_hydrogens (bool, default true)
  [output]       trajectory, energy_log (paths)
  [monitoring]   optional: energy_drift_threshold_kcal (f64), energy_drift_action ("warn" | "stop")

Additions (keys the reference does not know, so its parser rejects them):
  backend = "cuda"  the device-resident backend of this package;
  [cuda]         optional: precision ("mixed" | "fp64", default "mixed"),
                 frames_per_batch (u32 >= 1, default 64: trajectory frames the
                 device buffers between host reads), bonded_min_image (bool,
                 default false: with `periodic`, bonded, 1-4 and constraint
                 differences at the nearest image, which the reference leaves
                 raw);
  [[system]]     an array of system tables runs its systems as one batch in
                 one device context (gm_create_ensemble).  Each entry has the
                 [system] keys plus an optional `name` (default: its index);
                 the [output] paths take "{system}", replaced by the name, and
                 must contain it when the batch has more than one system.  The
                 systems of a batch share one box_size and periodic flag (one
                 gm_params) and the [run]/[integrator]/[nonbonded]/[constraints]
                 settings.

Errors are `ConfigError` with the reference's four kinds and messages
(geodesic-core/src/error.rs:65-79): a missing key gives MissingRequired with
the bare key name, an unknown key UnknownKey, a value of the wrong type or
range InvalidValue for key "config.toml" (config.rs:251-265), and the checks of
`validate` (config.rs:211-249) PhysicallyInvalid.  Keys are read in document
order and the first problem is reported, as serde does.
"""
from __future__ import annotations

import dataclasses
import enum
import math
import tomllib

_REQUIRED = object()


class ConfigError(ValueError):
    """ConfigError (geodesic-core/src/error.rs:65-79): `kind` is one of
    "UnknownKey", "InvalidValue", "MissingRequired", "PhysicallyInvalid"."""

    def __init__(self, kind: str, message: str, key: str = "", value: str = "", reason: str = ""):
        super().__init__(message)
        self.kind, self.key, self.value, self.reason = kind, key, value, reason

    @classmethod
    def unknown_key(cls, key):
        return cls("UnknownKey", f"unknown config key: {key}", key=key)

    @classmethod
    def invalid_value(cls, key, value, reason):
        return cls("InvalidValue", f"invalid value for key '{key}': '{value}' ({reason})", key=key, value=value,
                   reason=reason)

    @classmethod
    def missing_required(cls, key):
        return cls("MissingRequired", f"missing required config key: {key}", key=key)

    @classmethod
    def physically_invalid(cls, description):
        return cls("PhysicallyInvalid", f"physically invalid configuration: {description}", reason=description)


def _type_error(key, what):
    # a serde type or range error: InvalidValue on the whole file (config.rs:262-264)
    return ConfigError.invalid_value("config.toml", "", f"{key}: {what}")


def _kind(v) -> str:
    if isinstance(v, bool):
        return f"boolean `{str(v).lower()}`"
    if isinstance(v, int):
        return f"integer `{v}`"
    if isinstance(v, float):
        return f"floating point `{v!r}`"
    if isinstance(v, str):
        return f'string "{v}"'
    if isinstance(v, list):
        return "sequence"
    if isinstance(v, dict):
        return "map"
    return type(v).__name__


def _uint(bits, rust_name):
    hi = (1 << bits) - 1

    def conv(v, key):
        if isinstance(v, bool) or not isinstance(v, int):
            raise _type_error(key, f"invalid type: {_kind(v)}, expected {rust_name}")
        if v < 0 or v > hi:
            raise _type_error(key, f"invalid value: integer `{v}`, expected {rust_name}")
        return int(v)

    return conv


def _f64(v, key):
    # serde's f64 accepts TOML integers and floats
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise _type_error(key, f"invalid type: {_kind(v)}, expected f64")
    return float(v)


def _bool(v, key):
    if not isinstance(v, bool):
        raise _type_error(key, f"invalid type: {_kind(v)}, expected a boolean")
    return v


def _string(v, key):
    if not isinstance(v, str):
        raise _type_error(key, f"invalid type: {_kind(v)}, expected a string")
    return v


def _f64x3(v, key):
    if not isinstance(v, list):
        raise _type_error(key, f"invalid type: {_kind(v)}, expected an array of length 3")
    if len(v) != 3:
        raise _type_error(key, f"invalid length {len(v)}, expected an array of length 3")
    return tuple(_f64(x, key) for x in v)


def _struct(fields, what):
    """A serde struct with deny_unknown_fields: keys in document order (an
    unknown key or a bad value stops at once), then the first missing
    required field in declaration order."""
    names = dict(fields)

    def conv(table, key):
        if not isinstance(table, dict):
            raise _type_error(key, f"invalid type: {_kind(table)}, expected struct {what}")
        out = {}
        for k, v in table.items():
            f = names.get(k)
            if f is None:
                raise ConfigError.unknown_key(k)
            out[k] = f[0](v, k)
        for k, (_, default) in fields:
            if k not in out:
                if default is _REQUIRED:
                    raise ConfigError.missing_required(k)
                out[k] = default
        return out

    return conv


_RUN = _struct([("n_steps", (_uint(64, "u64"), _REQUIRED)), ("frame_interval", (_uint(32, "u32"), _REQUIRED)),
                ("backend", (_string, _REQUIRED)), ("n_threads", (_uint(64, "usize"), _REQUIRED))], "RawRun")
_SYSTEM_FIELDS = [("prmtop", (_string, _REQUIRED)), ("inpcrd", (_string, _REQUIRED)),
                  ("box_size", (_f64x3, _REQUIRED)), ("periodic", (_bool, False))]
_SYSTEM = _struct(_SYSTEM_FIELDS, "RawSystem")
_BATCH_ENTRY = _struct(_SYSTEM_FIELDS + [("name", (_string, None))], "RawSystem")
_INTEGRATOR = _struct([("dt", (_f64, _REQUIRED)), ("total_energy", (_f64, _REQUIRED))], "RawIntegrator")
_NONBONDED = _struct([("r_cutoff", (_f64, _REQUIRED)), ("r_skin", (_f64, _REQUIRED)),
                      ("r_switch", (_f64, _REQUIRED))], "RawNonbonded")
_CONSTRAINTS = _struct([("max_iter", (_uint(32, "u32"), _REQUIRED)), ("tolerance", (_f64, _REQUIRED)),
                        ("constrain_hydrogens", (_bool, True))], "RawConstraints")
_OUTPUT = _struct([("trajectory", (_string, _REQUIRED)), ("energy_log", (_string, _REQUIRED))], "RawOutput")
_MONITORING = _struct([("energy_drift_threshold_kcal", (_f64, _REQUIRED)),
                       ("energy_drift_action", (_string, _REQUIRED))], "RawMonitoring")
_CUDA = _struct([("precision", (_string, "mixed")), ("frames_per_batch", (_uint(32, "u32"), 64)),
                 ("bonded_min_image", (_bool, False))], "RawCuda")


def _system_or_batch(v, key):
    """`[system]` (one table, the reference's form) or `[[system]]` (an array
    of tables, a batch).  Returns (entries, is_batch)."""
    if isinstance(v, list):
        return [_BATCH_ENTRY(e, key) for e in v], True
    return [_SYSTEM(v, key)], False


_TOP = _struct([("run", (_RUN, _REQUIRED)), ("system", (_system_or_batch, _REQUIRED)),
                ("integrator", (_INTEGRATOR, _REQUIRED)), ("nonbonded", (_NONBONDED, _REQUIRED)),
                ("constraints", (_CONSTRAINTS, _REQUIRED)), ("output", (_OUTPUT, _REQUIRED)),
                ("monitoring", (_MONITORING, None)), ("cuda", (_CUDA, None))], "RawConfig")


class Backend(enum.Enum):
    """`[run].backend` (config.rs:82-90); `Cuda` is this package."""

    CPU = "cpu"
    GPU = "gpu"
    HYBRID = "hybrid"
    CUDA = "cuda"


class DriftAction(enum.Enum):
    WARN = "warn"
    STOP = "stop"


@dataclasses.dataclass(frozen=True)
class MonitoringConfig:
    energy_drift_threshold_kcal: float
    energy_drift_action: DriftAction


@dataclasses.dataclass(frozen=True)
class SystemConfig:
    """One `[system]` table: input files and box (config.rs:27-35)."""

    name: str
    prmtop: str
    inpcrd: str
    box_size: tuple
    periodic: bool


@dataclasses.dataclass
class Config:
    """Validated config.toml contents (config.rs:110-135).  `systems` holds
    one entry for the reference's `[system]` table (`batch` False) or the
    entries of a `[[system]]` array (`batch` True)."""

    n_steps: int
    frame_interval: int
    backend: Backend
    n_threads: int
    systems: list
    batch: bool
    dt: float
    total_energy: float
    r_cutoff: float
    r_skin: float
    r_switch: float
    max_constr_iter: int
    constr_tol: float
    constrain_hydrogens: bool
    trajectory: str
    energy_log: str
    monitoring: MonitoringConfig | None
    precision: str = "mixed"
    frames_per_batch: int = 64
    bonded_min_image: bool = False

    # the reference's single-system fields
    @property
    def prmtop(self) -> str:
        return self.systems[0].prmtop

    @property
    def inpcrd(self) -> str:
        return self.systems[0].inpcrd

    @property
    def box_size(self) -> tuple:
        return self.systems[0].box_size

    @property
    def periodic(self) -> bool:
        return self.systems[0].periodic

    @classmethod
    def from_toml_str(cls, s: str) -> "Config":
        """`Config::from_toml_str` (config.rs:138-208)."""
        try:
            doc = tomllib.loads(s)
        except tomllib.TOMLDecodeError as e:
            raise ConfigError.invalid_value("config.toml", "", str(e)) from None
        raw = _TOP(doc, "config.toml")
        run = raw["run"]
        try:
            backend = Backend(run["backend"])
        except ValueError:
            raise ConfigError.invalid_value("run.backend", run["backend"],
                                            'expected "cpu", "gpu", "hybrid", or "cuda"') from None
        monitoring = None
        if raw["monitoring"] is not None:
            m = raw["monitoring"]
            try:
                action = DriftAction(m["energy_drift_action"])
            except ValueError:
                raise ConfigError.invalid_value("monitoring.energy_drift_action", m["energy_drift_action"],
                                                'expected "warn" or "stop"') from None
            monitoring = MonitoringConfig(m["energy_drift_threshold_kcal"], action)
        entries, batch = raw["system"]
        systems = [SystemConfig(e.get("name") if e.get("name") is not None else str(k), e["prmtop"], e["inpcrd"],
                                e["box_size"], e["periodic"]) for k, e in enumerate(entries)]
        cuda = raw["cuda"] or {"precision": "mixed", "frames_per_batch": 64, "bonded_min_image": False}
        integ, nb, con, out = raw["integrator"], raw["nonbonded"], raw["constraints"], raw["output"]
        c = cls(n_steps=run["n_steps"], frame_interval=run["frame_interval"], backend=backend,
                n_threads=run["n_threads"], systems=systems, batch=batch, dt=integ["dt"],
                total_energy=integ["total_energy"], r_cutoff=nb["r_cutoff"], r_skin=nb["r_skin"],
                r_switch=nb["r_switch"], max_constr_iter=con["max_iter"], constr_tol=con["tolerance"],
                constrain_hydrogens=con["constrain_hydrogens"], trajectory=out["trajectory"],
                energy_log=out["energy_log"], monitoring=monitoring, precision=cuda["precision"],
                frames_per_batch=cuda["frames_per_batch"], bonded_min_image=cuda["bonded_min_image"])
        _validate(c)
        return c

    def outputs(self, k: int) -> tuple:
        """(trajectory, energy_log) paths of system k, before resolution
        against the config file's directory."""
        if not self.batch:
            return self.trajectory, self.energy_log
        name = self.systems[k].name
        return self.trajectory.replace("{system}", name), self.energy_log.replace("{system}", name)

    def sim_params(self):
        """The backend parameters of `into_sim_params` (config.rs:190-207)."""
        from . import backend as _be

        return _be.SimParams(box_size=tuple(self.box_size), periodic=self.periodic, r_cutoff=self.r_cutoff,
                             r_skin=self.r_skin, r_switch=self.r_switch, max_constr_iter=self.max_constr_iter,
                             constr_tol=self.constr_tol,
                             precision=_be.PRECISION_FP64 if self.precision == "fp64" else _be.PRECISION_MIXED,
                             bonded_min_image=self.bonded_min_image)


def _validate(c: Config) -> None:
    """`validate` (config.rs:211-249), in its order, then the checks of the
    additions."""
    if c.n_steps == 0:
        raise ConfigError.physically_invalid("run.n_steps must be greater than zero")
    for s in c.systems:
        if any(x <= 0.0 for x in s.box_size):
            raise ConfigError.physically_invalid("system.box_size components must be positive")
    if c.dt <= 0.0:
        raise ConfigError.physically_invalid("integrator.dt must be positive")
    if not (c.r_switch < c.r_cutoff and c.r_cutoff < c.r_skin):
        raise ConfigError.physically_invalid(
            "nonbonded radii must satisfy r_switch < r_cutoff < r_skin (got r_switch="
            f"{rust_f64(c.r_switch)}, r_cutoff={rust_f64(c.r_cutoff)}, r_skin={rust_f64(c.r_skin)})")
    if c.max_constr_iter == 0:
        raise ConfigError.physically_invalid("constraints.max_iter must be greater than zero")
    if c.constr_tol <= 0.0:
        raise ConfigError.physically_invalid("constraints.tolerance must be positive")

    if c.precision not in ("mixed", "fp64"):
        raise ConfigError.invalid_value("cuda.precision", c.precision, 'expected "mixed" or "fp64"')
    if not 1 <= c.frames_per_batch <= 2**31 - 1:
        raise ConfigError.invalid_value("cuda.frames_per_batch", str(c.frames_per_batch),
                                        "must be between 1 and 2^31 - 1")
    if not c.batch:
        return
    if not c.systems:
        raise ConfigError.invalid_value("system", "[]", "a batch needs at least one system")
    names = [s.name for s in c.systems]
    for k, nm in enumerate(names):
        if not nm or names.index(nm) != k:
            raise ConfigError.invalid_value("system.name", nm, "system names of a batch must be non-empty and unique")
    s0 = c.systems[0]
    for s in c.systems[1:]:
        if s.box_size != s0.box_size or s.periodic != s0.periodic:
            raise ConfigError.invalid_value("system.box_size", s.name,
                                            "the systems of a batch share one box_size and periodic flag")
    if len(c.systems) > 1:
        for key, path in (("output.trajectory", c.trajectory), ("output.energy_log", c.energy_log)):
            if "{system}" not in path:
                raise ConfigError.invalid_value(key, path, 'a batch of several systems needs "{system}" in the path')


def rust_f64(x: float) -> str:
    """An f64 as Rust's `{}` prints it: the shortest digits that read back
    to the same value, positional, no trailing `.0` ("12", "0.0001", "NaN")."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    r = repr(float(x))
    if "e" not in r and "E" not in r:
        return r[:-2] if r.endswith(".0") else r
    mant, exp = r.split("e")
    sign = "-" if mant.startswith("-") else ""
    mant = mant.lstrip("-")
    digits = mant.replace(".", "")
    point = (mant.index(".") if "." in mant else len(mant)) + int(exp)
    if point <= 0:
        s = "0." + "0" * (-point) + digits
    elif point >= len(digits):
        s = digits + "0" * (point - len(digits))
    else:
        s = digits[:point] + "." + digits[point:]
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return sign + s


def load(path: str) -> Config:
    """Reads and validates a config file (the first half of
    `run_from_config_file`, geodesic/src/lib.rs:175-180)."""
    with open(path, encoding="utf-8") as f:
        return Config.from_toml_str(f.read())
