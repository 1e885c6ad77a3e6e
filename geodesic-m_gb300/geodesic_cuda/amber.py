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


def _field_bytes(sections: dict, flag: str, width: int, count: int):
    """The `count` fixed-width fields of a section as a numpy byte-string
    array, or None when the section is not plain ASCII (the per-field path
    then keeps the reference's character positions)."""
    if flag not in sections:
        raise PrmtopError(f"missing required config key: %FLAG {flag}")
    raw = sections[flag]
    if not raw.isascii():
        return None
    need = width * count
    # a field past the end of the data parses as blank (an error), a partly
    # present one as its characters, as in the per-field path
    b = raw[:need].encode("ascii").ljust(need)
    return np.frombuffer(b, dtype=f"S{width}")


def _ints_np(sections, flag, width, count) -> np.ndarray:
    """`_ints` for whole sections at once; any field the vectorised parse
    rejects goes through `_ints`, which raises the reference's error."""
    f = _field_bytes(sections, flag, width, count)
    try:
        if f is not None:
            return f.astype(np.int64)
    except ValueError:
        pass
    return np.asarray(_ints(sections, flag, width, count), np.int64)


def _floats_np(sections, flag, width, count) -> np.ndarray:
    f = _field_bytes(sections, flag, width, count)
    try:
        if f is not None:
            return f.astype(np.float64)
    except ValueError:
        pass
    return np.asarray(_floats(sections, flag, width, count), np.float64)


def _elements(names: np.ndarray) -> np.ndarray:
    """`infer_element` for an (N,) array of 4-byte names: the first ASCII
    letter decides."""
    b = np.frombuffer(names.tobytes(), np.uint8).reshape(-1, 4) if len(names) else np.zeros((0, 4), np.uint8)
    upper = b & 0xDF  # ASCII letters to upper case
    alpha = ((b >= 65) & (b <= 90)) | ((b >= 97) & (b <= 122))
    has = alpha.any(axis=1)
    first = upper[np.arange(len(b)), alpha.argmax(axis=1)] if len(b) else np.zeros(0, np.uint8)
    out = np.full(len(b), ELEMENT_UNKNOWN, np.uint8)
    for ch, el in ((b"H", ELEMENT_H), (b"C", ELEMENT_C), (b"N", ELEMENT_N), (b"O", ELEMENT_O), (b"S", ELEMENT_S)):
        out[has & (first == ch[0])] = el
    return out


def parse_prmtop(text: str) -> tuple:
    """Returns (AtomData, BondedTopology) like `prmtop::parse` (`prmtop.rs:182`).

    Whole sections are parsed as numpy fixed-width arrays (a million-atom
    file in seconds); the per-atom and per-term assembly is vectorised with
    the reference's exact rules."""
    s = _sections(text)
    p = _ints(s, "POINTERS", 8, 20)
    natom, ntypes, nbonh, ntheth, nphih = p[0], p[1], p[2], p[4], p[6]
    nnb, nres, nbona, ntheta, nphia = p[10], p[11], p[12], p[13], p[14]
    numbnd, numang, nptra = p[15], p[16], p[17]

    names_b = _field_bytes(s, "ATOM_NAME", 4, natom)
    if names_b is None:
        names = _fields(s, "ATOM_NAME", 4, natom)
        element = np.array([infer_element(n) for n in names], np.uint8)
    else:
        names = [n.decode("ascii") for n in names_b]
        element = _elements(names_b)
    charge = _floats_np(s, "CHARGE", 16, natom) / AMBER_CHARGE_TO_ELEMENTARY
    mass = _floats_np(s, "MASS", 16, natom)
    type_index = _ints_np(s, "ATOM_TYPE_INDEX", 8, natom)
    n_excluded = _ints_np(s, "NUMBER_EXCLUDED_ATOMS", 8, natom)
    nb_index = _ints_np(s, "NONBONDED_PARM_INDEX", 8, ntypes * ntypes)
    n_lj = ntypes * (ntypes + 1) // 2
    acoef = _floats_np(s, "LENNARD_JONES_ACOEF", 16, n_lj)
    bcoef = _floats_np(s, "LENNARD_JONES_BCOEF", 16, n_lj)
    res_ptr = _ints_np(s, "RESIDUE_POINTER", 8, nres)
    excl_list = _ints_np(s, "EXCLUDED_ATOMS_LIST", 8, nnb)

    # per type (prmtop.rs:216-237), then per atom; the first atom of a 10-12
    # type is the one reported
    ico = nb_index[ntypes * (type_index - 1) + type_index - 1] if natom else np.zeros(0, np.int64)
    bad = np.nonzero(ico <= 0)[0]
    if len(bad):
        i = int(bad[0])
        raise PrmtopError(f"atom {i} uses a 10-12 H-bond LJ type (NONBONDED_PARM_INDEX={int(ico[i])}); not supported")
    sig_t, eps_t = {}, {}
    for c in np.unique(ico):
        a, b = float(acoef[c - 1]), float(bcoef[c - 1])
        if a == 0.0 or b == 0.0:
            sig_t[c] = eps_t[c] = 0.0
        else:
            sig_t[c] = math.pow(a / b, 1.0 / 6.0)
            eps_t[c] = (b * b) / (4.0 * a)
    uniq, inv = np.unique(ico, return_inverse=True)
    sigma = np.array([sig_t[c] for c in uniq], np.float64)[inv] if natom else np.zeros(0)
    epsilon = np.array([eps_t[c] for c in uniq], np.float64)[inv] if natom else np.zeros(0)

    # residue of atom i: the last pointer before the first one past i + 1
    # (the reference's scan breaks there), i.e. a search in the running maximum
    if nres:
        cummax = np.maximum.accumulate(res_ptr)
        residue = np.maximum(np.searchsorted(cummax, np.arange(1, natom + 1), side="right") - 1, 0)
    else:
        residue = np.zeros(natom, np.int64)
    atoms = AtomData(sigma, epsilon, mass, charge, element, residue.astype(np.uint32), [n.ljust(4) for n in names])

    raw_b = np.concatenate([_ints_np(s, "BONDS_INC_HYDROGEN", 8, 3 * nbonh),
                            _ints_np(s, "BONDS_WITHOUT_HYDROGEN", 8, 3 * nbona)]).reshape(-1, 3)
    raw_a = np.concatenate([_ints_np(s, "ANGLES_INC_HYDROGEN", 8, 4 * ntheth),
                            _ints_np(s, "ANGLES_WITHOUT_HYDROGEN", 8, 4 * ntheta)]).reshape(-1, 4)
    raw_d = np.concatenate([_ints_np(s, "DIHEDRALS_INC_HYDROGEN", 8, 5 * nphih),
                            _ints_np(s, "DIHEDRALS_WITHOUT_HYDROGEN", 8, 5 * nphia)]).reshape(-1, 5)
    bk = _floats_np(s, "BOND_FORCE_CONSTANT", 16, numbnd)
    br0 = _floats_np(s, "BOND_EQUIL_VALUE", 16, numbnd)
    ak = _floats_np(s, "ANGLE_FORCE_CONSTANT", 16, numang)
    ath0 = _floats_np(s, "ANGLE_EQUIL_VALUE", 16, numang)
    dk = _floats_np(s, "DIHEDRAL_FORCE_CONSTANT", 16, nptra)
    dper = _floats_np(s, "DIHEDRAL_PERIODICITY", 16, nptra)
    dphase = _floats_np(s, "DIHEDRAL_PHASE", 16, nptra)
    bt = raw_b[:, 2] - 1
    at = raw_a[:, 3] - 1
    dt = raw_d[:, 4] - 1
    abs_d = np.abs(raw_d)

    # exclusions in list order, one run per atom, 0 entries skipped
    # (prmtop.rs:303-317)
    total = int(n_excluded.sum()) if natom else 0
    if total > len(excl_list) or (natom and n_excluded.min() < 0):
        raise PrmtopError(f"invalid value for key '%FLAG NUMBER_EXCLUDED_ATOMS': the counts ask for {total} "
                          f"entries of EXCLUDED_ATOMS_LIST, which has {len(excl_list)}")
    owner = np.repeat(np.arange(natom, dtype=np.int64), n_excluded) if natom else np.zeros(0, np.int64)
    raw_e = excl_list[:total]
    keep = raw_e != 0

    per = dper[dt]
    u32 = lambda a: np.asarray(a, np.uint32)  # noqa: E731
    topo = BondedTopology(
        bond_i=u32(raw_b[:, 0] // 3), bond_j=u32(raw_b[:, 1] // 3),
        bond_k=bk[bt].astype(np.float64), bond_r0=br0[bt].astype(np.float64),
        angle_i=u32(raw_a[:, 0] // 3), angle_j=u32(raw_a[:, 1] // 3), angle_k=u32(raw_a[:, 2] // 3),
        angle_kth=ak[at].astype(np.float64), angle_th0=ath0[at].astype(np.float64),
        dihed_i=u32(abs_d[:, 0] // 3), dihed_j=u32(abs_d[:, 1] // 3), dihed_k=u32(abs_d[:, 2] // 3),
        dihed_l=u32(abs_d[:, 3] // 3), dihed_kphi=dk[dt].astype(np.float64),
        dihed_n=u32((np.floor(np.abs(per) + 0.5) * np.where(per >= 0, 1.0, -1.0)).astype(np.int64)),
        dihed_delta=dphase[dt].astype(np.float64),
        constr_i=u32([]), constr_j=u32([]), constr_dsq=np.zeros(0),
        excl_i=u32(owner[keep]), excl_j=u32(raw_e[keep] - 1))
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
        if txt.isascii():
            try:
                return np.frombuffer(txt[:nval * 12].encode("ascii").ljust(nval * 12), dtype="S12").astype(np.float64)
            except ValueError:
                pass
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
