"""Writes a parsed or synthetic system back out as AMBER prmtop / inpcrd
text, in the layout `geodesic_cuda.amber` (and the reference's readers,
prmtop.rs:182-344, inpcrd.rs:26-98) read: one Lennard-Jones type per distinct
(sigma, epsilon), one bond / angle / dihedral parameter type per term, 10-atom
residues, `%16.8E` reals and `%12.7f` coordinates.  Reading the files back
gives the system to within those formats' rounding; tests compare runs on
what the files hold, so the rounding does not matter."""
import numpy as np

from geodesic_cuda.amber import AMBER_CHARGE_TO_ELEMENTARY, AMBER_VELOCITY_TO_ANG_PER_PS, ELEMENT_H

_SYMBOL = {0: "H", 1: "C", 2: "N", 3: "O", 4: "S"}


def _block(flag, fmt, values, per_line, conv):
    lines = [f"%FLAG {flag}", f"%FORMAT({fmt})"]
    vals = list(values)
    for k in range(0, len(vals), per_line):
        lines.append("".join(conv(v) for v in vals[k:k + per_line]))
    if not vals:
        lines.append("")
    return lines


def prmtop_text(atoms, topo) -> str:
    n = atoms.n
    key = list(zip(atoms.sigma.tolist(), atoms.epsilon.tolist()))
    kinds = sorted(set(key))
    type_of = {k: t for t, k in enumerate(kinds)}
    types = [type_of[k] + 1 for k in key]
    nt = len(kinds)
    # triangular A/B tables; only the diagonal entries define an atom's sigma and epsilon
    nb_index = [max(i, j) * (max(i, j) - 1) // 2 + min(i, j) for i in range(1, nt + 1) for j in range(1, nt + 1)]
    acoef, bcoef = [], []
    for hi in range(nt):
        for lo in range(hi + 1):
            s = 0.5 * (kinds[hi][0] + kinds[lo][0])
            e = (kinds[hi][1] * kinds[lo][1]) ** 0.5
            acoef.append(4.0 * e * s ** 12)
            bcoef.append(4.0 * e * s ** 6)
    is_h = atoms.element == ELEMENT_H
    names = [(_SYMBOL.get(int(el), "X") + str(i % 1000)).ljust(4)[:4] for i, el in enumerate(atoms.element)]

    nb, na, nd = len(topo.bond_i), len(topo.angle_i), len(topo.dihed_i)
    bonds = [(int(topo.bond_i[t]), int(topo.bond_j[t]), t + 1) for t in range(nb)]
    angles = [(int(topo.angle_i[t]), int(topo.angle_j[t]), int(topo.angle_k[t]), t + 1) for t in range(na)]
    diheds = [(int(topo.dihed_i[t]), int(topo.dihed_j[t]), int(topo.dihed_k[t]), int(topo.dihed_l[t]), t + 1)
              for t in range(nd)]
    b_h = [b for b in bonds if is_h[b[0]] or is_h[b[1]]]
    b_a = [b for b in bonds if not (is_h[b[0]] or is_h[b[1]])]
    a_h = [a for a in angles if is_h[a[0]] or is_h[a[1]] or is_h[a[2]]]
    a_a = [a for a in angles if not (is_h[a[0]] or is_h[a[1]] or is_h[a[2]])]
    d_h = [d for d in diheds if any(is_h[x] for x in d[:4])]
    d_a = [d for d in diheds if not any(is_h[x] for x in d[:4])]
    excl = [[] for _ in range(n)]
    for i, j in zip(topo.excl_i.tolist(), topo.excl_j.tolist()):
        excl[i].append(j + 1)
    excl = [e or [0] for e in excl]
    nres = (n + 9) // 10

    ptr = [0] * 31
    ptr[0], ptr[1], ptr[2], ptr[3], ptr[4], ptr[5] = n, nt, len(b_h), len(b_a), len(a_h), len(a_a)
    ptr[6], ptr[7], ptr[10], ptr[11] = len(d_h), len(d_a), sum(len(e) for e in excl), nres
    ptr[12], ptr[13], ptr[14], ptr[15], ptr[16], ptr[17] = len(b_a), len(a_a), len(d_a), max(nb, 1), max(na, 1), \
        max(nd, 1)
    e16 = lambda v: f"{float(v):16.8E}"  # noqa: E731
    i8 = lambda v: f"{int(v):8d}"  # noqa: E731
    flat = lambda rows, k: [x * 3 if c < k else x for r in rows for c, x in enumerate(r)]  # noqa: E731
    pad = lambda a: list(a) if len(a) else [0.0]  # noqa: E731
    lines = ["%VERSION  VERSION_STAMP = V0001.000", "%FLAG TITLE", "%FORMAT(20a4)", "written by tests/amber_files.py"]
    lines += _block("POINTERS", "10I8", ptr, 10, i8)
    lines += _block("ATOM_NAME", "20a4", names, 20, str)
    lines += _block("CHARGE", "5E16.8", atoms.charge * AMBER_CHARGE_TO_ELEMENTARY, 5, e16)
    lines += _block("MASS", "5E16.8", atoms.mass, 5, e16)
    lines += _block("ATOM_TYPE_INDEX", "10I8", types, 10, i8)
    lines += _block("NUMBER_EXCLUDED_ATOMS", "10I8", [len(e) for e in excl], 10, i8)
    lines += _block("NONBONDED_PARM_INDEX", "10I8", nb_index, 10, i8)
    lines += _block("RESIDUE_POINTER", "10I8", [1 + 10 * r for r in range(nres)], 10, i8)
    lines += _block("BOND_FORCE_CONSTANT", "5E16.8", pad(topo.bond_k), 5, e16)
    lines += _block("BOND_EQUIL_VALUE", "5E16.8", pad(topo.bond_r0), 5, e16)
    lines += _block("ANGLE_FORCE_CONSTANT", "5E16.8", pad(topo.angle_kth), 5, e16)
    lines += _block("ANGLE_EQUIL_VALUE", "5E16.8", pad(topo.angle_th0), 5, e16)
    lines += _block("DIHEDRAL_FORCE_CONSTANT", "5E16.8", pad(topo.dihed_kphi), 5, e16)
    lines += _block("DIHEDRAL_PERIODICITY", "5E16.8", pad(topo.dihed_n), 5, e16)
    lines += _block("DIHEDRAL_PHASE", "5E16.8", pad(topo.dihed_delta), 5, e16)
    lines += _block("LENNARD_JONES_ACOEF", "5E16.8", acoef, 5, e16)
    lines += _block("LENNARD_JONES_BCOEF", "5E16.8", bcoef, 5, e16)
    lines += _block("BONDS_INC_HYDROGEN", "10I8", flat(b_h, 2), 10, i8)
    lines += _block("BONDS_WITHOUT_HYDROGEN", "10I8", flat(b_a, 2), 10, i8)
    lines += _block("ANGLES_INC_HYDROGEN", "10I8", flat(a_h, 3), 10, i8)
    lines += _block("ANGLES_WITHOUT_HYDROGEN", "10I8", flat(a_a, 3), 10, i8)
    lines += _block("DIHEDRALS_INC_HYDROGEN", "10I8", flat(d_h, 4), 10, i8)
    lines += _block("DIHEDRALS_WITHOUT_HYDROGEN", "10I8", flat(d_a, 4), 10, i8)
    lines += _block("EXCLUDED_ATOMS_LIST", "10I8", [x for e in excl for x in e], 10, i8)
    return "\n".join(lines) + "\n"


def inpcrd_text(pos, vel) -> str:
    n = pos.shape[1]
    lines = ["written by tests/amber_files.py", f"{n:6d}"]
    for block in (pos.T.reshape(-1), (vel / AMBER_VELOCITY_TO_ANG_PER_PS).T.reshape(-1)):
        for k in range(0, 3 * n, 6):
            lines.append("".join(f"{v:12.7f}" for v in block[k:k + 6]))
    return "\n".join(lines) + "\n"


def write_system(directory, stem, atoms, topo, state):
    """Writes <stem>.prmtop and <stem>.inpcrd; returns their file names."""
    prm, crd = f"{stem}.prmtop", f"{stem}.inpcrd"
    (directory / prm).write_text(prmtop_text(atoms, topo))
    (directory / crd).write_text(inpcrd_text(np.asarray(state.pos), np.asarray(state.vel)))
    return prm, crd
