"""Fast prmtop/inpcrd ingest (whole sections parsed as numpy fixed-width
arrays) against a field-by-field restatement of `prmtop.rs:182-344` and
`inpcrd.rs:26-98`, on seeded synthetic AMBER files: identical arrays, bit
for bit, the reference's errors on bad input, and a 200,000-atom file read
in seconds (CPU only)."""
import math
import time

import numpy as np
import pytest

from geodesic_cuda import amber
from geodesic_cuda.amber import (AMBER_CHARGE_TO_ELEMENTARY, AtomData, BondedTopology, PrmtopError, _fields,
                                 _floats, _ints, _round_half_away, _sections, infer_element)


def per_field_prmtop(text: str) -> tuple:
    """The field-by-field restatement of `prmtop::parse` (`prmtop.rs:182`)."""
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


def _block(flag, fmt, values, per_line, width, conv):
    lines = [f"%FLAG {flag}", f"%FORMAT({fmt})"]
    vals = list(values)
    for k in range(0, len(vals), per_line):
        lines.append("".join(conv(v).rjust(width) if width else conv(v) for v in vals[k:k + per_line]))
    if not vals:
        lines.append("")
    return lines


def synthetic_prmtop(n, seed):
    """A chain of n atoms in AMBER prmtop layout: 8 LJ types, ~30 % hydrogens,
    bonds/angles/dihedrals along the chain (split into the with/without H
    sections), 1-2/1-3/1-4 exclusions, residues of 10 atoms."""
    rng = np.random.default_rng(seed)
    nt = 8
    is_h = rng.random(n) < 0.3
    names = [("H" if h else "C") + str(i % 100) for i, h in enumerate(is_h)]
    types = rng.integers(1, nt + 1, n)
    charge = rng.uniform(-0.5, 0.5, n) * 18.2223
    mass = np.where(is_h, 1.008, rng.uniform(12.0, 16.0, n))
    bonds = [(i, i + 1, 1 + i % 5) for i in range(n - 1)]
    angles = [(i, i + 1, i + 2, 1 + i % 4) for i in range(n - 2)]
    diheds = [(i, i + 1, (-1 if i % 7 == 0 else 1) * (i + 2), i + 3, 1 + i % 3) for i in range(n - 3)]
    excl = [[j + 1 for j in range(i + 1, min(i + 4, n))] or [0] for i in range(n)]
    hb = lambda t: is_h[t[0]] or is_h[t[1]]  # noqa: E731
    b_h = [b for b in bonds if hb(b)]
    b_a = [b for b in bonds if not hb(b)]
    a_h = [a for a in angles if is_h[a[0]] or is_h[a[1]] or is_h[a[2]]]
    a_a = [a for a in angles if not (is_h[a[0]] or is_h[a[1]] or is_h[a[2]])]
    d_h = [d for d in diheds if is_h[d[0]] or is_h[d[1]] or is_h[abs(d[2])] or is_h[d[3]]]
    d_a = [d for d in diheds if not (is_h[d[0]] or is_h[d[1]] or is_h[abs(d[2])] or is_h[d[3]])]
    nres = (n + 9) // 10
    ptr = [0] * 31
    ptr[0], ptr[1], ptr[2], ptr[4], ptr[6] = n, nt, len(b_h), len(a_h), len(d_h)
    ptr[10], ptr[11], ptr[12], ptr[13], ptr[14] = sum(len(e) for e in excl), nres, len(b_a), len(a_a), len(d_a)
    ptr[15], ptr[16], ptr[17] = 5, 4, 3
    # index of the type pair in the triangular A/B tables (1-based)
    nb_index = [max(i, j) * (max(i, j) - 1) // 2 + min(i, j) for i in range(1, nt + 1) for j in range(1, nt + 1)]
    n_lj = nt * (nt + 1) // 2
    sig = rng.uniform(2.0, 3.8, n_lj)
    eps = rng.uniform(0.02, 0.2, n_lj)
    acoef = 4 * eps * sig ** 12
    bcoef = 4 * eps * sig ** 6
    acoef[3] = 0.0  # a type pair without LJ (sigma = epsilon = 0)
    e16 = lambda v: f"{v:16.8E}"  # noqa: E731
    i8 = lambda v: f"{int(v):8d}"  # noqa: E731
    flat = lambda rows, k: [x * 3 if c < k else x for r in rows for c, x in enumerate(r)]  # noqa: E731
    lines = ["%VERSION  VERSION_STAMP = V0001.000", "%FLAG TITLE", "%FORMAT(20a4)", "synthetic"]
    lines += _block("POINTERS", "10I8", ptr, 10, 8, str)
    lines += _block("ATOM_NAME", "20a4", names, 20, 0, lambda s: s.ljust(4)[:4])
    lines += _block("CHARGE", "5E16.8", charge, 5, 0, e16)
    lines += _block("MASS", "5E16.8", mass, 5, 0, e16)
    lines += _block("ATOM_TYPE_INDEX", "10I8", types, 10, 0, i8)
    lines += _block("NUMBER_EXCLUDED_ATOMS", "10I8", [len(e) for e in excl], 10, 0, i8)
    lines += _block("NONBONDED_PARM_INDEX", "10I8", nb_index, 10, 0, i8)
    lines += _block("RESIDUE_POINTER", "10I8", [1 + 10 * r for r in range(nres)], 10, 0, i8)
    lines += _block("BOND_FORCE_CONSTANT", "5E16.8", [300.0, 340.0, 250.5, 410.0, 367.0], 5, 0, e16)
    lines += _block("BOND_EQUIL_VALUE", "5E16.8", [1.09, 1.52, 1.33, 1.01, 1.41], 5, 0, e16)
    lines += _block("ANGLE_FORCE_CONSTANT", "5E16.8", [50.0, 63.0, 35.0, 80.0], 5, 0, e16)
    lines += _block("ANGLE_EQUIL_VALUE", "5E16.8", [1.91, 2.09, 1.88, 2.0], 5, 0, e16)
    lines += _block("DIHEDRAL_FORCE_CONSTANT", "5E16.8", [0.15, 1.4, 0.25], 5, 0, e16)
    lines += _block("DIHEDRAL_PERIODICITY", "5E16.8", [3.0, 2.0, 1.0], 5, 0, e16)
    lines += _block("DIHEDRAL_PHASE", "5E16.8", [0.0, 3.14159265, 0.0], 5, 0, e16)
    lines += _block("LENNARD_JONES_ACOEF", "5E16.8", acoef, 5, 0, e16)
    lines += _block("LENNARD_JONES_BCOEF", "5E16.8", bcoef, 5, 0, e16)
    lines += _block("BONDS_INC_HYDROGEN", "10I8", flat(b_h, 2), 10, 0, i8)
    lines += _block("BONDS_WITHOUT_HYDROGEN", "10I8", flat(b_a, 2), 10, 0, i8)
    lines += _block("ANGLES_INC_HYDROGEN", "10I8", flat(a_h, 3), 10, 0, i8)
    lines += _block("ANGLES_WITHOUT_HYDROGEN", "10I8", flat(a_a, 3), 10, 0, i8)
    lines += _block("DIHEDRALS_INC_HYDROGEN", "10I8", flat(d_h, 4), 10, 0, i8)
    lines += _block("DIHEDRALS_WITHOUT_HYDROGEN", "10I8", flat(d_a, 4), 10, 0, i8)
    lines += _block("EXCLUDED_ATOMS_LIST", "10I8", [x for e in excl for x in e], 10, 0, i8)
    return "\n".join(lines) + "\n"


def synthetic_inpcrd(n, seed, with_vel=True):
    rng = np.random.default_rng(seed)
    vals = list(rng.uniform(-50, 50, 3 * n)) + (list(rng.uniform(-1, 1, 3 * n)) if with_vel else [])
    lines = ["synthetic", f"{n:6d}"]
    for k in range(0, 3 * n, 6):
        lines.append("".join(f"{v:12.7f}" for v in vals[k:min(k + 6, 3 * n)]))
    if with_vel:
        for k in range(3 * n, 6 * n, 6):
            lines.append("".join(f"{v:12.7f}" for v in vals[k:min(k + 6, 6 * n)]))
    return "\n".join(lines) + "\n"


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes()


@pytest.mark.parametrize("n,seed", [(1, 3), (37, 4), (1003, 5)])
def test_fast_prmtop_equals_per_field_restatement(n, seed):
    text = synthetic_prmtop(n, seed)
    fa, ft = amber.parse_prmtop(text)
    ra, rt = per_field_prmtop(text)
    for f in ("sigma", "epsilon", "mass", "charge", "element", "residue_id"):
        assert same(getattr(fa, f), getattr(ra, f)), f
    assert list(fa.names) == list(ra.names)
    for f in ("bond_i", "bond_j", "bond_k", "bond_r0", "angle_i", "angle_j", "angle_k", "angle_kth", "angle_th0",
              "dihed_i", "dihed_j", "dihed_k", "dihed_l", "dihed_kphi", "dihed_n", "dihed_delta", "excl_i", "excl_j"):
        assert same(getattr(ft, f), getattr(rt, f)), f


def test_fast_inpcrd_equals_per_field():
    text = synthetic_inpcrd(1001, 9)
    st = amber.parse_inpcrd(text, 1001)
    vals = np.array([float(x) for line in text.splitlines()[2:] for x in (line[i:i + 12] for i in range(0, len(line), 12))])
    assert np.array_equal(st.pos, vals[:3003].reshape(1001, 3).T)
    assert np.array_equal(st.vel, vals[3003:].reshape(1001, 3).T * 20.455)


def test_bad_fields_raise_the_reference_errors():
    text = synthetic_prmtop(30, 6)
    bad = text.replace("%FLAG MASS\n%FORMAT(5E16.8)\n", "%FLAG MASS\n%FORMAT(5E16.8)\n   not-a-number!",
                       1)
    with pytest.raises(PrmtopError, match="FLAG MASS"):
        amber.parse_prmtop(bad)
    with pytest.raises(PrmtopError, match="missing required config key: %FLAG CHARGE"):
        amber.parse_prmtop(text.replace("%FLAG CHARGE", "%FLAG CHARGEX"))


def test_large_file_reads_in_seconds():
    n = 200_000
    text = synthetic_prmtop(n, 7)
    t0 = time.perf_counter()
    atoms, topo = amber.parse_prmtop(text)
    dt = time.perf_counter() - t0
    assert atoms.n == n and len(topo.dihed_i) == n - 3 and len(topo.excl_i) == 3 * n - 6
    assert dt < 10.0, dt
