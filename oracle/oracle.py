"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the CPU restatement of the reference engine in `oracle.c`; this
module wraps it for the tests, the smoke check and the CPU-baseline leg of the
bench.  Nothing in the CUDA backend imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_u32p = C.POINTER(C.c_uint32)
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)
_u8p = C.POINTER(C.c_uint8)


class OrAtoms(C.Structure):
    _fields_ = [("n", C.c_int64), ("sigma", _f64p), ("epsilon", _f64p), ("mass", _f64p),
                ("charge", _f64p), ("element", _u8p)]


class OrTopology(C.Structure):
    _fields_ = [("n_bonds", C.c_int64), ("bond_i", _u32p), ("bond_j", _u32p), ("bond_k", _f64p), ("bond_r0", _f64p),
                ("n_angles", C.c_int64), ("angle_i", _u32p), ("angle_j", _u32p), ("angle_k", _u32p),
                ("angle_kth", _f64p), ("angle_th0", _f64p),
                ("n_diheds", C.c_int64), ("dihed_i", _u32p), ("dihed_j", _u32p), ("dihed_k", _u32p),
                ("dihed_l", _u32p), ("dihed_kphi", _f64p), ("dihed_n", _u32p), ("dihed_delta", _f64p),
                ("n_constr", C.c_int64), ("constr_i", _u32p), ("constr_j", _u32p), ("constr_dsq", _f64p),
                ("n_excl", C.c_int64), ("excl_i", _u32p), ("excl_j", _u32p)]


class OrParams(C.Structure):
    _fields_ = [("box", C.c_double * 3), ("periodic", C.c_int32), ("n_threads", C.c_int32),
                ("r_cutoff", C.c_double), ("r_skin", C.c_double), ("r_switch", C.c_double),
                ("max_constr_iter", C.c_uint32), ("constr_tol", C.c_double),
                ("coulomb", C.c_int32), ("scale14_lj", C.c_double), ("scale14_coul", C.c_double),
                ("bonded_min_image", C.c_int32)]


class OrConvergenceError(C.Structure):
    _fields_ = [("step", C.c_uint64), ("constraint_idx", C.c_int64), ("atom_i", C.c_int64),
                ("atom_j", C.c_int64), ("residual", C.c_double), ("max_iter", C.c_uint32)]


class ConvergenceError(RuntimeError):
    """ConvergenceError::ConstraintSolver (geodesic-core/src/error.rs:50-63)."""

    def __init__(self, e: OrConvergenceError):
        self.step, self.constraint_idx = int(e.step), int(e.constraint_idx)
        self.atom_i, self.atom_j = int(e.atom_i), int(e.atom_j)
        self.residual, self.max_iter = float(e.residual), int(e.max_iter)
        super().__init__(f"constraint solver failed to converge for constraint {self.constraint_idx} "
                         f"(atoms {self.atom_i}, {self.atom_j}) at step {self.step}: residual "
                         f"{self.residual} after {self.max_iter} iterations")


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.POINTER
        L.or_neighbor_build.restype = C.c_int64
        L.or_neighbor_build.argtypes = [C.c_int64, _f64p, _f64p, _f64p, P(OrParams), P(OrTopology), C.c_int64, _u32p, _u32p]
        L.or_neighbor_build_cells.restype = C.c_int64
        L.or_neighbor_build_cells.argtypes = L.or_neighbor_build.argtypes
        L.or_neighbor_pairs.restype = C.c_int64
        L.or_neighbor_pairs.argtypes = L.or_neighbor_build.argtypes + [C.c_int32]
        L.or_needs_rebuild.restype = C.c_int32
        L.or_needs_rebuild.argtypes = [C.c_int64] + [_f64p] * 6 + [C.c_double, C.c_double]
        for name in ("or_pair_forces", "or_coulomb_forces"):
            f = getattr(L, name)
            f.restype = C.c_double
            f.argtypes = [_f64p, _f64p, _f64p, P(OrAtoms), _u32p, _u32p, C.c_int64, C.c_double, C.c_double,
                          _f64p, _f64p, _f64p, _f64p]
        L.or_pairs14.restype = C.c_int64
        L.or_pairs14.argtypes = [P(OrTopology), C.c_int64, C.c_int64, _u32p, _u32p]
        L.or_pair14_forces.restype = C.c_double
        L.or_pair14_forces.argtypes = [_f64p, _f64p, _f64p, P(OrAtoms), _u32p, _u32p, C.c_int64, C.c_double,
                                       C.c_double, C.c_int32, _f64p, _f64p, _f64p]
        for name in ("or_bond_forces", "or_angle_forces", "or_dihedral_forces"):
            f = getattr(L, name)
            f.restype = C.c_double
            f.argtypes = [_f64p, _f64p, _f64p, P(OrTopology), _f64p, _f64p, _f64p]
            f = getattr(L, name + "_box")
            f.restype = C.c_double
            f.argtypes = [_f64p, _f64p, _f64p, P(OrTopology), _f64p, _f64p, _f64p, _f64p]
        L.or_pair14_forces_box.restype = C.c_double
        L.or_pair14_forces_box.argtypes = [_f64p, _f64p, _f64p, P(OrAtoms), _u32p, _u32p, C.c_int64, C.c_double,
                                           C.c_double, C.c_int32, _f64p, _f64p, _f64p, _f64p]
        L.or_constraint_solve_box.restype = C.c_int64
        L.or_constraint_solve_box.argtypes = [P(OrTopology), P(OrAtoms)] + [_f64p] * 6 + [
            C.c_uint32, C.c_double, C.c_uint64, _f64p, _f64p, _f64p, P(OrConvergenceError)]
        L.or_constrain_velocities_box.restype = C.c_int64
        L.or_constrain_velocities_box.argtypes = [P(OrTopology), P(OrAtoms)] + [_f64p] * 6 + [
            C.c_uint32, C.c_double, C.c_uint64, _f64p, P(OrConvergenceError)]
        L.or_drift_and_constrain_box.restype = C.c_int64
        L.or_drift_and_constrain_box.argtypes = [C.c_int64] + [_f64p] * 6 + [
            P(OrTopology), P(OrAtoms), C.c_double, C.c_uint32, C.c_double, C.c_uint64, _f64p, P(OrConvergenceError)]
        L.or_constraint_solve_ws.restype = C.c_int64
        L.or_constraint_solve_ws.argtypes = [P(OrTopology), P(OrAtoms), _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                             C.c_uint32, C.c_double, C.c_uint64, _f64p, _f64p, P(OrConvergenceError)]
        L.or_constrain_velocities.restype = C.c_int64
        L.or_constrain_velocities.argtypes = [P(OrTopology), P(OrAtoms), _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                              C.c_uint32, C.c_double, C.c_uint64, P(OrConvergenceError)]
        L.or_half_kick.restype = None
        L.or_half_kick.argtypes = [C.c_int64] + [_f64p] * 7 + [C.c_double]
        L.or_drift_and_constrain.restype = C.c_int64
        L.or_drift_and_constrain.argtypes = [C.c_int64] + [_f64p] * 6 + [P(OrTopology), P(OrAtoms), C.c_double,
                                                                         C.c_uint32, C.c_double, C.c_uint64,
                                                                         P(OrConvergenceError)]
        L.or_kinetic_energy.restype = C.c_double
        L.or_kinetic_energy.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _f64p]
        L.or_backend_new.restype = C.c_void_p
        L.or_backend_new.argtypes = [P(OrAtoms), P(OrTopology), P(OrParams)]
        L.or_backend_free.argtypes = [C.c_void_p]
        L.or_backend_n_threads.restype = C.c_int32
        L.or_backend_n_threads.argtypes = [C.c_void_p]
        L.or_backend_build_neighbor_list.restype = C.c_int64
        L.or_backend_build_neighbor_list.argtypes = [C.c_void_p, _f64p, _f64p, _f64p]
        L.or_backend_pairs.restype = C.c_int64
        L.or_backend_pairs.argtypes = [C.c_void_p, P(_u32p), P(_u32p)]
        L.or_backend_set_pairs.restype = C.c_int64
        L.or_backend_set_pairs.argtypes = [C.c_void_p, C.c_int64, _u32p, _u32p, _f64p, _f64p, _f64p]
        L.or_backend_compute_forces.restype = C.c_double
        L.or_backend_compute_forces.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p]
        L.or_backend_needs_rebuild.restype = C.c_int32
        L.or_backend_needs_rebuild.argtypes = [C.c_void_p, _f64p, _f64p, _f64p]
        L.or_backend_geodesic_drift.restype = C.c_int64
        L.or_backend_geodesic_drift.argtypes = [C.c_void_p] + [_f64p] * 6 + [C.c_double, C.c_uint64,
                                                                             P(OrConvergenceError)]
        L.or_run.restype = C.c_int64
        L.or_run.argtypes = [P(OrAtoms), P(OrTopology), P(OrParams)] + [_f64p] * 6 + [
            C.c_double, C.c_uint64, C.c_uint32, C.c_int64, _f32p, _f64p, _f64p, C.POINTER(C.c_uint64),
            P(OrConvergenceError)]
        L.or_host_threads.restype = C.c_int32
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Arrays:
    """Keeps contiguous copies alive while C holds pointers into them."""

    def __init__(self, atoms, topo):
        n = int(len(atoms.mass))
        self.keep = []

        def f(a):
            a = _f64(a)
            self.keep.append(a)
            return _p(a, C.c_double)

        def u(a):
            a = _u32(a)
            self.keep.append(a)
            return _p(a, C.c_uint32)

        el = np.ascontiguousarray(getattr(atoms, "element", np.full(n, 5, np.uint8)), dtype=np.uint8)
        self.keep.append(el)
        charge = getattr(atoms, "charge", np.zeros(n))
        self.atoms = OrAtoms(n, f(atoms.sigma), f(atoms.epsilon), f(atoms.mass), f(charge), _p(el, C.c_uint8))
        t = topo
        self.topo = OrTopology(
            len(t.bond_i), u(t.bond_i), u(t.bond_j), f(t.bond_k), f(t.bond_r0),
            len(t.angle_i), u(t.angle_i), u(t.angle_j), u(t.angle_k), f(t.angle_kth), f(t.angle_th0),
            len(t.dihed_i), u(t.dihed_i), u(t.dihed_j), u(t.dihed_k), u(t.dihed_l), f(t.dihed_kphi),
            u(t.dihed_n), f(t.dihed_delta),
            len(t.constr_i), u(t.constr_i), u(t.constr_j), f(t.constr_dsq),
            len(t.excl_i), u(t.excl_i), u(t.excl_j))


def make_params(box=(1000.0, 1000.0, 1000.0), periodic=False, r_cutoff=12.0, r_skin=14.0, r_switch=10.0,
                max_constr_iter=100, constr_tol=1e-10, n_threads=1, coulomb=False, scale14_lj=0.0,
                scale14_coul=0.0, bonded_min_image=False):
    return OrParams((C.c_double * 3)(*box), int(periodic), int(n_threads), r_cutoff, r_skin, r_switch,
                    int(max_constr_iter), constr_tol, int(coulomb), scale14_lj, scale14_coul, int(bonded_min_image))


def _box(box):
    """The nearest-image box of the *_box functions (None: raw differences)."""
    if box is None:
        return None, None
    b = np.ascontiguousarray(box, dtype=np.float64)
    return b, _p(b, C.c_double)


def host_threads() -> int:
    return int(lib().or_host_threads())


def neighbor_build(pos, atoms, topo, params, cells=False):
    """neighbor::build: wraps pos in place (periodic) and returns (pair_i, pair_j)."""
    L = lib()
    arr = Arrays(atoms, topo)
    n = pos.shape[1]
    assert pos.dtype == np.float64 and pos.flags.c_contiguous
    fn = L.or_neighbor_build_cells if cells else L.or_neighbor_build
    px, py, pz = (_p(pos[d], C.c_double) for d in range(3))
    cnt = fn(n, px, py, pz, C.byref(params), C.byref(arr.topo), 0, None, None)
    pi = np.zeros(max(cnt, 1), np.uint32)
    pj = np.zeros(max(cnt, 1), np.uint32)
    # the positions are wrapped now: the fill call does not wrap again
    cnt2 = L.or_neighbor_pairs(n, px, py, pz, C.byref(params), C.byref(arr.topo), cnt, _p(pi, C.c_uint32),
                               _p(pj, C.c_uint32), int(cells))
    assert cnt2 == cnt
    return pi[:cnt].copy(), pj[:cnt].copy()


def needs_rebuild(pos, ref, r_skin, r_cutoff) -> bool:
    return bool(lib().or_needs_rebuild(pos.shape[1], *(_p(_f64(pos[d]), C.c_double) for d in range(3)),
                                       *(_p(_f64(ref[d]), C.c_double) for d in range(3)), r_skin, r_cutoff))


def _forces_call(fname, pos, atoms, pair_i, pair_j, r_cutoff, r_switch, box, force=None):
    L = lib()
    arr = Arrays(atoms, _empty_topo())
    n = pos.shape[1]
    force = np.zeros((3, n)) if force is None else force
    pi, pj = _u32(pair_i), _u32(pair_j)
    b = (C.c_double * 3)(*box)
    e = getattr(L, fname)(*(_p(_f64(pos[d]), C.c_double) for d in range(3)), C.byref(arr.atoms),
                          _p(pi, C.c_uint32), _p(pj, C.c_uint32), len(pi), r_cutoff, r_switch, b,
                          *(_p(force[d], C.c_double) for d in range(3)))
    return e, force


def pair_forces(pos, atoms, pair_i, pair_j, r_cutoff, r_switch, box=(1000.0,) * 3, force=None):
    """force::nonbonded::compute_pair_forces -> (energy, force (3, N))."""
    return _forces_call("or_pair_forces", pos, atoms, pair_i, pair_j, r_cutoff, r_switch, box, force)


def coulomb_forces(pos, atoms, pair_i, pair_j, r_cutoff, r_switch, box=(1000.0,) * 3, force=None):
    return _forces_call("or_coulomb_forces", pos, atoms, pair_i, pair_j, r_cutoff, r_switch, box, force)


def pairs14(topo, n_atoms):
    L = lib()
    arr = Arrays(_dummy_atoms(n_atoms), topo)
    cnt = L.or_pairs14(C.byref(arr.topo), n_atoms, 0, None, None)
    pi = np.zeros(max(cnt, 1), np.uint32)
    pj = np.zeros(max(cnt, 1), np.uint32)
    L.or_pairs14(C.byref(arr.topo), n_atoms, cnt, _p(pi, C.c_uint32), _p(pj, C.c_uint32))
    return pi[:cnt].copy(), pj[:cnt].copy()


def pair14_forces(pos, atoms, p14_i, p14_j, scale_lj, scale_coul, coulomb, force=None, box=None):
    L = lib()
    arr = Arrays(atoms, _empty_topo())
    n = pos.shape[1]
    force = np.zeros((3, n)) if force is None else force
    pi, pj = _u32(p14_i), _u32(p14_j)
    keep, bp = _box(box)
    e = L.or_pair14_forces_box(*(_p(_f64(pos[d]), C.c_double) for d in range(3)), C.byref(arr.atoms),
                               _p(pi, C.c_uint32), _p(pj, C.c_uint32), len(pi), scale_lj, scale_coul, int(coulomb),
                               bp, *(_p(force[d], C.c_double) for d in range(3)))
    return e, force


def bonded_forces(kind, pos, topo, force=None, box=None):
    """kind in {'bond', 'angle', 'dihedral'} -> (energy, force); `box`: the
    nearest-image box of the *_box variants."""
    L = lib()
    n = pos.shape[1]
    arr = Arrays(_dummy_atoms(n), topo)
    force = np.zeros((3, n)) if force is None else force
    if box is None:
        fn = {"bond": L.or_bond_forces, "angle": L.or_angle_forces, "dihedral": L.or_dihedral_forces}[kind]
        e = fn(*(_p(_f64(pos[d]), C.c_double) for d in range(3)), C.byref(arr.topo),
               *(_p(force[d], C.c_double) for d in range(3)))
        return e, force
    fn = {"bond": L.or_bond_forces_box, "angle": L.or_angle_forces_box, "dihedral": L.or_dihedral_forces_box}[kind]
    keep, bp = _box(box)
    e = fn(*(_p(_f64(pos[d]), C.c_double) for d in range(3)), C.byref(arr.topo), bp,
           *(_p(force[d], C.c_double) for d in range(3)))
    return e, force


def constraint_solve(topo, atoms, ref, pos, max_iter, tol, step=0, lam0=None, want_lambda=False):
    """constraint::solve; modifies pos in place. Returns iterations (and summed
    multipliers when want_lambda); raises ConvergenceError."""
    L = lib()
    arr = Arrays(atoms, topo)
    err = OrConvergenceError()
    refc = _f64(ref)
    lam_out = np.zeros(len(topo.constr_i)) if want_lambda else None
    l0 = _f64(lam0) if lam0 is not None else None
    it = L.or_constraint_solve_ws(C.byref(arr.topo), C.byref(arr.atoms), *(_p(refc[d], C.c_double) for d in range(3)),
                                  *(_p(pos[d], C.c_double) for d in range(3)), max_iter, tol, step,
                                  _p(l0, C.c_double) if l0 is not None else None,
                                  _p(lam_out, C.c_double) if lam_out is not None else None, C.byref(err))
    if it < 0:
        raise ConvergenceError(err)
    return (int(it), lam_out) if want_lambda else int(it)


def constrain_velocities(topo, atoms, pos, vel, max_iter, tol, step=0, box=None):
    L = lib()
    arr = Arrays(atoms, topo)
    err = OrConvergenceError()
    posc = _f64(pos)
    keep, bp = _box(box)
    it = L.or_constrain_velocities_box(C.byref(arr.topo), C.byref(arr.atoms),
                                       *(_p(posc[d], C.c_double) for d in range(3)),
                                       *(_p(vel[d], C.c_double) for d in range(3)), max_iter, tol, step, bp,
                                       C.byref(err))
    if it < 0:
        raise ConvergenceError(err)
    return int(it)


def half_kick(vel, force, mass, dt_half):
    L = lib()
    fc, m = _f64(force), _f64(mass)
    L.or_half_kick(vel.shape[1], *(_p(vel[d], C.c_double) for d in range(3)), *(_p(fc[d], C.c_double) for d in range(3)),
                   _p(m, C.c_double), dt_half)


def drift_and_constrain(pos, vel, topo, atoms, dt, max_iter, tol, step=0, box=None):
    L = lib()
    arr = Arrays(atoms, topo)
    err = OrConvergenceError()
    keep, bp = _box(box)
    it = L.or_drift_and_constrain_box(pos.shape[1], *(_p(pos[d], C.c_double) for d in range(3)),
                                      *(_p(vel[d], C.c_double) for d in range(3)), C.byref(arr.topo),
                                      C.byref(arr.atoms), dt, max_iter, tol, step, bp, C.byref(err))
    if it < 0:
        raise ConvergenceError(err)
    return int(it)


def drift_and_constrain_ws(pos, vel, topo, atoms, dt, max_iter, tol, lam0, step=0):
    """integrator.rs:32-71 with the SHAKE warm start of constraint_solve
    (lam0: predicted multipliers applied once before the iterations).  The
    same operations as or_drift_and_constrain.  Returns (iterations, summed
    multipliers)."""
    ref = pos.copy()
    pos += dt * vel
    it, lam = constraint_solve(topo, atoms, ref, pos, max_iter, tol, step, lam0=lam0, want_lambda=True)
    vel[...] = (pos - ref) / dt
    return it, lam


def kinetic_energy(vel, mass) -> float:
    m = _f64(mass)
    v = _f64(vel)
    return float(lib().or_kinetic_energy(v.shape[1], *(_p(v[d], C.c_double) for d in range(3)), _p(m, C.c_double)))


class CpuBackend:
    """CpuBackend (geodesic-engine/src/cpu_backend.rs:25-219) on the oracle."""

    def __init__(self, atoms, topo, params):
        self._arr = Arrays(atoms, topo)
        self._params = params
        self.n = int(len(atoms.mass))
        self._h = lib().or_backend_new(C.byref(self._arr.atoms), C.byref(self._arr.topo), C.byref(params))
        self.potential_energy = 0.0

    def __del__(self):
        if getattr(self, "_h", None):
            lib().or_backend_free(self._h)
            self._h = None

    def n_threads(self) -> int:
        return int(lib().or_backend_n_threads(self._h))

    def build_neighbor_list(self, pos) -> int:
        return int(lib().or_backend_build_neighbor_list(self._h, *(_p(pos[d], C.c_double) for d in range(3))))

    def pairs(self):
        pi, pj = _u32p(), _u32p()
        cnt = lib().or_backend_pairs(self._h, C.byref(pi), C.byref(pj))
        if cnt == 0:
            return np.zeros(0, np.uint32), np.zeros(0, np.uint32)
        return (np.ctypeslib.as_array(pi, shape=(cnt,)).copy(), np.ctypeslib.as_array(pj, shape=(cnt,)).copy())

    def set_pairs(self, pair_i, pair_j, pos):
        """Installs the given pair list (the reference's set) and build positions."""
        pi, pj, p = _u32(pair_i), _u32(pair_j), _f64(pos)
        lib().or_backend_set_pairs(self._h, len(pi), _p(pi, C.c_uint32), _p(pj, C.c_uint32),
                                   *(_p(p[d], C.c_double) for d in range(3)))

    def compute_forces(self, pos):
        f = np.zeros((3, self.n))
        p = _f64(pos)
        self.potential_energy = float(lib().or_backend_compute_forces(
            self._h, *(_p(p[d], C.c_double) for d in range(3)), *(_p(f[d], C.c_double) for d in range(3))))
        return f

    def needs_rebuild(self, pos) -> bool:
        p = _f64(pos)
        return bool(lib().or_backend_needs_rebuild(self._h, *(_p(p[d], C.c_double) for d in range(3))))

    def geodesic_drift(self, pos, vel, dt, step=0) -> int:
        err = OrConvergenceError()
        it = lib().or_backend_geodesic_drift(self._h, *(_p(pos[d], C.c_double) for d in range(3)),
                                             *(_p(vel[d], C.c_double) for d in range(3)), dt, step, C.byref(err))
        if it < 0:
            raise ConvergenceError(err)
        return int(it)


def run(atoms, topo, params, pos, vel, dt, n_steps, frame_interval=1):
    """geodesic/src/lib.rs:187-333 -> (frames float32 (F,3,N), pot, kin)."""
    L = lib()
    arr = Arrays(atoms, topo)
    n = pos.shape[1]
    max_frames = n_steps // frame_interval + 1
    frames = np.zeros((max_frames, 3, n), np.float32)
    pot = np.zeros(max_frames)
    kin = np.zeros(max_frames)
    fail = C.c_uint64()
    err = OrConvergenceError()
    rc = L.or_run(C.byref(arr.atoms), C.byref(arr.topo), C.byref(params), *(_p(pos[d], C.c_double) for d in range(3)),
                  *(_p(vel[d], C.c_double) for d in range(3)), dt, n_steps, frame_interval, max_frames,
                  _p(frames, C.c_float), _p(pot, C.c_double), _p(kin, C.c_double), C.byref(fail), C.byref(err))
    if rc == -1:
        raise ConvergenceError(err)
    if rc < 0:
        raise FloatingPointError(f"non-finite {'force' if rc == -2 else 'position'} at step {fail.value}")
    return frames[:rc], pot[:rc], kin[:rc]


class _Obj:
    pass


def _dummy_atoms(n):
    a = _Obj()
    a.sigma = a.epsilon = a.charge = np.zeros(n)
    a.mass = np.ones(n)
    a.element = np.full(n, 5, np.uint8)
    return a


def _empty_topo():
    t = _Obj()
    for k in ("bond_i", "bond_j", "angle_i", "angle_j", "angle_k", "dihed_i", "dihed_j", "dihed_k", "dihed_l",
              "dihed_n", "constr_i", "constr_j", "excl_i", "excl_j"):
        setattr(t, k, np.zeros(0, np.uint32))
    for k in ("bond_k", "bond_r0", "angle_kth", "angle_th0", "dihed_kphi", "dihed_delta", "constr_dsq"):
        setattr(t, k, np.zeros(0))
    return t
