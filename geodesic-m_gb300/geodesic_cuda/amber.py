"""AMBER prmtop / inpcrd ingest for the CUDA backend.

These readers produce exactly the inputs the reference's engine receives:
`AtomData` (per-atom sigma, epsilon, mass, charge, element) and
`BondedTopology` (bonds, angles, dihedrals, constraints, exclusions), all as
numpy arrays in the reference's SoA layout.  The semantics follow
`geodesic-io/src/prmtop.rs:182-344` and `geodesic-io/src/inpcrd.rs:26-98`:

* sections are keyed by `%FLAG` and hold the concatenation of their data
  lines, sliced into fixed-width fields (`fixed_width.rs:4-14`);
* per-atom sigma = (A/B)^(1/6) and epsilon = B^2/(4A) come from the diagonal
  `NONBONDED_PARM_INDEX` entry of the atom's type; A == 0 or B == 0 gives
  sigma = epsilon = 0 (`prmtop.rs:216-237`);
* CHARGE is divided by 18.2223 (`prmtop.rs:9,201-205`);
* bond/angle/dihedral atom indices are the stored value / 3; dihedral entries
  take abs() first (`prmtop.rs:138-180`); dihedral multiplicity is rounded
  (`prmtop.rs:297-300`);
* exclusions come from `EXCLUDED_ATOMS_LIST` with 0 entries skipped
  (`prmtop.rs:303-317`);
* the element is inferred from the first alphabetic character of the atom
  name (`prmtop.rs:102-117`); only hydrogen matters on the hot path (H-bond
  promotion, `constraint.rs:21-22`).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

AMBER_CHARGE_TO_ELEMENTARY = 18.2223
AMBER_VELOCITY_TO_ANG_PER_PS = 20.455

ELEMENT_H, ELEMENT_C, ELEMENT_N, ELEMENT_O, ELEMENT_S, ELEMENT_UNKNOWN = range(6)


class PrmtopError(ValueError):
    """Raised for the reference's ConfigError cases (missing section, bad field,
    unsupported 10-12 LJ type, atom-count mismatch)."""


@dataclasses.dataclass
class AtomData:
    """Per-atom parameters, `geodesic-core/src/atoms.rs:3-12`."""

    sigma: np.ndarray
    epsilon: np.ndarray
    mass: np.ndarray
    charge: np.ndarray
    element: np.ndarray  # uint8, ELEMENT_* codes
    residue_id: np.ndarray
    names: list

    @property
    def n(self) -> int:
        return int(self.mass.shape[0])


@dataclasses.dataclass
class BondedTopology:
    """Connectivity, `geodesic-core/src/topology.rs:4-37` (SoA, uint32 indices)."""

    bond_i: np.ndarray
    bond_j: np.ndarray
    bond_k: np.ndarray
    bond_r0: np.ndarray
    angle_i: np.ndarray
    angle_j: np.ndarray
    angle_k: np.ndarray
    angle_kth: np.ndarray
    angle_th0: np.ndarray
    dihed_i: np.ndarray
    dihed_j: np.ndarray
    dihed_k: np.ndarray
    dihed_l: np.ndarray
    dihed_kphi: np.ndarray
    dihed_n: np.ndarray
    dihed_delta: np.ndarray
    constr_i: np.ndarray
    constr_j: np.ndarray
    constr_dsq: np.ndarray
    excl_i: np.ndarray
    excl_j: np.ndarray

    @staticmethod
    def empty() -> "BondedTopology":
        u = lambda: np.zeros(0, np.uint32)  # noqa: E731
        f = lambda: np.zeros(0, np.float64)  # noqa: E731
        return BondedTopology(u(), u(), f(), f(), u(), u(), u(), f(), f(), u(), u(), u(), u(),
                              f(), u(), f(), u(), u(), f(), u(), u())

    def copy(self) -> "BondedTopology":
        return BondedTopology(**{k: np.array(v, copy=True) for k, v in dataclasses.asdict(self).items()})


@dataclasses.dataclass
class State:
    """Positions (A) and velocities (A/ps), `geodesic-core/src/state.rs:3-23`."""

    pos: np.ndarray  # (3, N) float64: rows x, y, z
    vel: np.ndarray  # (3, N) float64


def _sections(text: str) -> dict:
    """`prmtop.rs:16-47`: concatenated data text per %FLAG, directives skipped."""
    sections: dict = {}
    current = None
    for line in text.splitlines():
        if line.startswith("%FLAG "):
            current = line[len("%FLAG "):].strip()
            sections.setdefault(current, [])
            continue
        if line.startswith("%"):
            continue
        if current is not None:
            sections[current].append(line)
    return {k: "".join(v) for k, v in sections.items()}


def _fields(sections: dict, flag: str, width: int, count: int) -> list:
    """`fixed_width.rs:4-14`: `count` fields of exactly `width` characters."""
    if flag not in sections:
        raise PrmtopError(f"missing required config key: %FLAG {flag}")
    raw = sections[flag]
    out = []
    for i in range(count):
        start = i * width
        out.append(raw[start:start + width] if start < len(raw) else "")
    return out


def _ints(sections, flag, width, count):
    vals = []
    for f in _fields(sections, flag, width, count):
        try:
            vals.append(int(f.strip()))
        except ValueError as e:
            raise PrmtopError(f"invalid value for key '%FLAG {flag}': '{f}' (expected an integer)") from e
    return vals


def _floats(sections, flag, width, count):
    vals = []
    for f in _fields(sections, flag, width, count):
        try:
            vals.append(float(f.strip()))
        except ValueError as e:
            raise PrmtopError(f"invalid value for key '%FLAG {flag}': '{f}' (expected a float)") from e
    return vals


def infer_element(name: str) -> int:
    """`prmtop.rs:102-117`."""
    for c in name:
        if c.isascii() and c.isalpha():
            return {"H": ELEMENT_H, "C": ELEMENT_C, "N": ELEMENT_N, "O": ELEMENT_O,
                    "S": ELEMENT_S}.get(c.upper(), ELEMENT_UNKNOWN)
    return ELEMENT_UNKNOWN


def parse_prmtop(text: str) -> tuple:
    """Returns (AtomData, BondedTopology) like `prmtop::parse` (`prmtop.rs:182`)."""
    s = _sections(text)
    p = _ints(s, "POINTERS", 8, 20)
    natom, ntypes, nbonh, ntheth, nphih = p[0], p[1], p[2], p[4], p[6]
    nnb, nres, nbona, ntheta, nphia = p[10], p[11], p[12], p[13], p[14]
    numbnd, numang, nptra = p[15], p[16], p[17]

    names = _fields(s, "ATOM_NAME", 4, natom)
    charge = np.array(_floats(s, "CHARGE", 16, natom), np.float64) / AMBER_CHARGE_TO_ELEMENTARY
    mass = np.array(_floats(s, "MASS", 16, natom), np.float64)
    type_index = _ints(s, "ATOM_TYPE_INDEX", 8, natom)
    n_excluded = _ints(s, "NUMBER_EXCLUDED_ATOMS", 8, natom)
    nb_index = _ints(s, "NONBONDED_PARM_INDEX", 8, ntypes * ntypes)
    n_lj = ntypes * (ntypes + 1) // 2
    acoef = _floats(s, "LENNARD_JONES_ACOEF", 16, n_lj)
    bcoef = _floats(s, "LENNARD_JONES_BCOEF", 16, n_lj)
    res_ptr = _ints(s, "RESIDUE_POINTER", 8, nres)
    excl_list = _ints(s, "EXCLUDED_ATOMS_LIST", 8, nnb)

    sigma = np.zeros(natom)
    epsilon = np.zeros(natom)
    for i, ty in enumerate(type_index):
        ico = nb_index[ntypes * (ty - 1) + ty - 1]
        if ico <= 0:
            raise PrmtopError(f"atom {i} uses a 10-12 H-bond LJ type (NONBONDED_PARM_INDEX={ico}); not supported")
        a, b = acoef[ico - 1], bcoef[ico - 1]
        if a == 0.0 or b == 0.0:
            sigma[i] = epsilon[i] = 0.0
        else:
            sigma[i] = math.pow(a / b, 1.0 / 6.0)
            epsilon[i] = (b * b) / (4.0 * a)

    element = np.array([infer_element(n) for n in names], np.uint8)
    residue = np.zeros(natom, np.uint32)
    for i in range(natom):
        rid = 0
        for r, start in enumerate(res_ptr):
            if start <= i + 1:
                rid = r
            else:
                break
        residue[i] = rid
    atoms = AtomData(sigma, epsilon, mass, charge, element, residue, [n.ljust(4) for n in names])

    bonds_h = _ints(s, "BONDS_INC_HYDROGEN", 8, 3 * nbonh)
    bonds_a = _ints(s, "BONDS_WITHOUT_HYDROGEN", 8, 3 * nbona)
    angles_h = _ints(s, "ANGLES_INC_HYDROGEN", 8, 4 * ntheth)
    angles_a = _ints(s, "ANGLES_WITHOUT_HYDROGEN", 8, 4 * ntheta)
    dihed_h = _ints(s, "DIHEDRALS_INC_HYDROGEN", 8, 5 * nphih)
    dihed_a = _ints(s, "DIHEDRALS_WITHOUT_HYDROGEN", 8, 5 * nphia)
    bk = _floats(s, "BOND_FORCE_CONSTANT", 16, numbnd)
    br0 = _floats(s, "BOND_EQUIL_VALUE", 16, numbnd)
    ak = _floats(s, "ANGLE_FORCE_CONSTANT", 16, numang)
    ath0 = _floats(s, "ANGLE_EQUIL_VALUE", 16, numang)
    dk = _floats(s, "DIHEDRAL_FORCE_CONSTANT", 16, nptra)
    dper = _floats(s, "DIHEDRAL_PERIODICITY", 16, nptra)
    dphase = _floats(s, "DIHEDRAL_PHASE", 16, nptra)

    raw_b = np.array(bonds_h + bonds_a, np.int64).reshape(-1, 3)
    raw_a = np.array(angles_h + angles_a, np.int64).reshape(-1, 4)
    raw_d = np.abs(np.array(dihed_h + dihed_a, np.int64).reshape(-1, 5))
    bt = raw_b[:, 2] - 1
    at = raw_a[:, 3] - 1
    dt = np.array(dihed_h + dihed_a, np.int64).reshape(-1, 5)[:, 4] - 1

    excl_i, excl_j = [], []
    cursor = 0
    for i, cnt in enumerate(n_excluded):
        for _ in range(cnt):
            raw = excl_list[cursor]
            cursor += 1
            if raw == 0:
                continue
            excl_i.append(i)
            excl_j.append(raw - 1)

    f64 = lambda a: np.asarray(a, np.float64)  # noqa: E731
    u32 = lambda a: np.asarray(a, np.uint32)  # noqa: E731
    topo = BondedTopology(
        bond_i=u32(raw_b[:, 0] // 3), bond_j=u32(raw_b[:, 1] // 3),
        bond_k=f64([bk[t] for t in bt]), bond_r0=f64([br0[t] for t in bt]),
        angle_i=u32(raw_a[:, 0] // 3), angle_j=u32(raw_a[:, 1] // 3), angle_k=u32(raw_a[:, 2] // 3),
        angle_kth=f64([ak[t] for t in at]), angle_th0=f64([ath0[t] for t in at]),
        dihed_i=u32(raw_d[:, 0] // 3), dihed_j=u32(raw_d[:, 1] // 3), dihed_k=u32(raw_d[:, 2] // 3),
        dihed_l=u32(raw_d[:, 3] // 3), dihed_kphi=f64([dk[t] for t in dt]),
        dihed_n=u32([_round_half_away(dper[t]) for t in dt]), dihed_delta=f64([dphase[t] for t in dt]),
        constr_i=u32([]), constr_j=u32([]), constr_dsq=f64([]),
        excl_i=u32(excl_i), excl_j=u32(excl_j))
    return atoms, topo


def _round_half_away(x: float) -> int:
    """Rust `f64::round` (half away from zero)."""
    return int(math.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)


def parse_inpcrd(text: str, expected_n_atoms: int, has_box: bool = False) -> State:
    """`inpcrd.rs:26-98`: 6F12.7 coordinates, optional velocity block (x20.455)."""
    lines = text.splitlines()
    if len(lines) < 2:
        raise PrmtopError("file has fewer than 2 lines (missing title or atom-count header)")
    natom = int(lines[1].split()[0])
    if natom != expected_n_atoms:
        raise PrmtopError(f"inpcrd declares {natom} atoms but prmtop declares {expected_n_atoms}")
    nval = natom * 3
    nlines = (nval + 5) // 6
    data = lines[2:]
    if len(data) < nlines:
        raise PrmtopError(f"expected {nlines} coordinate line(s) for {natom} atoms, found {len(data)}")

    def block(txt):
        return np.array([float(txt[i * 12:(i + 1) * 12].strip()) for i in range(nval)], np.float64)

    pos = block("".join(data[:nlines])).reshape(natom, 3).T.copy()
    vel = np.zeros_like(pos)
    remaining = data[nlines:]
    avail = max(len(remaining) - (1 if has_box else 0), 0)
    if avail >= nlines and nlines > 0:
        vel = block("".join(remaining[:nlines])).reshape(natom, 3).T.copy() * AMBER_VELOCITY_TO_ANG_PER_PS
    return State(pos=pos, vel=vel)


def promote_hydrogen_bonds(topo: BondedTopology, atoms: AtomData) -> BondedTopology:
    """`constraint.rs:10-40`: bonds touching an H atom become constraints
    (dsq = r0^2), the rest stay harmonic; both keep their original order."""
    t = topo.copy()
    h = atoms.element == ELEMENT_H
    touch = h[t.bond_i] | h[t.bond_j]
    r0 = t.bond_r0[touch]
    t.constr_i = np.concatenate([t.constr_i, t.bond_i[touch]]).astype(np.uint32)
    t.constr_j = np.concatenate([t.constr_j, t.bond_j[touch]]).astype(np.uint32)
    t.constr_dsq = np.concatenate([t.constr_dsq, r0 * r0])
    keep = ~touch
    t.bond_i, t.bond_j = t.bond_i[keep], t.bond_j[keep]
    t.bond_k, t.bond_r0 = t.bond_k[keep], t.bond_r0[keep]
    return t


def load(prmtop_path: str, inpcrd_path: str, has_box: bool = False):
    with open(prmtop_path) as f:
        atoms, topo = parse_prmtop(f.read())
    with open(inpcrd_path) as f:
        state = parse_inpcrd(f.read(), atoms.n, has_box)
    return atoms, topo, state


def save_npz(path: str, atoms: AtomData, topo: BondedTopology, state: State, **extra) -> None:
    """Stores a parsed system as plain arrays (no pickles)."""
    arrays = {f"atoms_{k}": v for k, v in dataclasses.asdict(atoms).items() if k != "names"}
    arrays["atoms_names"] = np.array(atoms.names, dtype="U4")
    arrays.update({f"topo_{k}": v for k, v in dataclasses.asdict(topo).items()})
    arrays["pos"] = state.pos
    arrays["vel"] = state.vel
    arrays.update(extra)
    np.savez_compressed(path, **arrays)


def load_npz(path: str):
    """Inverse of `save_npz`: returns (AtomData, BondedTopology, State, extras)."""
    z = np.load(path, allow_pickle=False)
    a = {f.name: z[f"atoms_{f.name}"] for f in dataclasses.fields(AtomData) if f.name != "names"}
    atoms = AtomData(names=[str(s) for s in z["atoms_names"]], **a)
    topo = BondedTopology(**{f.name: z[f"topo_{f.name}"] for f in dataclasses.fields(BondedTopology)})
    state = State(pos=z["pos"].copy(), vel=z["vel"].copy())
    known = {f"atoms_{f.name}" for f in dataclasses.fields(AtomData)} | {
        f"topo_{f.name}" for f in dataclasses.fields(BondedTopology)} | {"pos", "vel"}
    extra = {k: z[k] for k in z.files if k not in known}
    return atoms, topo, state, extra
