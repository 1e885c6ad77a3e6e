"""Python host mirror of the reference's `ComputeBackend` trait over the C ABI.

`CudaBackend` has the trait's methods with the same meaning
(geodesic-core/src/backend.rs:11-23): it owns the atoms and topology, keeps
the neighbour list and forces on the GPU, and returns forces in the reference
layout (three float64 rows of N).  The engine free functions the run loop
calls directly (integrator::half_kick, constraint::constrain_velocities and
the kinetic-energy sum of lib.rs:68-77) are methods here too, so a run loop
can drive the whole step through this object.

There is no CPU fallback: constructing a backend without the compiled
library or without a CUDA device raises `BackendError`.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

from . import _build

GM_OK = 0
GM_ERR_INVALID_ARGUMENT = 1
STATUS_NAMES = {
    1: "INVALID_ARGUMENT", 2: "NO_DEVICE", 3: "OUT_OF_MEMORY", 4: "DEVICE", 5: "CONVERGENCE", 6: "NONFINITE",
    7: "LIST_OVERFLOW", 8: "UNSUPPORTED", 9: "FIXED_POINT_OVERFLOW", 10: "NOT_BUILT",
}
PRECISION_MIXED, PRECISION_FP64 = 0, 1
STEP_GRAPH, STEP_PERSISTENT = 0, 1  # gm_step_form

_u32p = C.POINTER(C.c_uint32)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


class BackendError(RuntimeError):
    """BackendError (geodesic-core/src/error.rs:81-91) and the other status codes."""

    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class NumericalError(BackendError):
    """NumericalError (error.rs:34-48): non-finite force or position."""


class ConvergenceError(BackendError):
    """ConvergenceError::ConstraintSolver (error.rs:50-63)."""

    def __init__(self, status, message, conv):
        super().__init__(status, message)
        self.step, self.constraint_idx = int(conv.step), int(conv.constraint_idx)
        self.atom_i, self.atom_j = int(conv.atom_i), int(conv.atom_j)
        self.residual, self.max_iter = float(conv.residual), int(conv.max_iter)


class GmAtoms(C.Structure):
    _fields_ = [("n_atoms", C.c_int64), ("sigma", _f64p), ("epsilon", _f64p), ("mass", _f64p),
                ("charge", _f64p), ("element", _u8p)]


class GmTopology(C.Structure):
    _fields_ = [("n_bonds", C.c_int64), ("bond_i", _u32p), ("bond_j", _u32p), ("bond_k", _f64p), ("bond_r0", _f64p),
                ("n_angles", C.c_int64), ("angle_i", _u32p), ("angle_j", _u32p), ("angle_k", _u32p),
                ("angle_kth", _f64p), ("angle_th0", _f64p),
                ("n_diheds", C.c_int64), ("dihed_i", _u32p), ("dihed_j", _u32p), ("dihed_k", _u32p),
                ("dihed_l", _u32p), ("dihed_kphi", _f64p), ("dihed_n", _u32p), ("dihed_delta", _f64p),
                ("n_constr", C.c_int64), ("constr_i", _u32p), ("constr_j", _u32p), ("constr_dsq", _f64p),
                ("n_excl", C.c_int64), ("excl_i", _u32p), ("excl_j", _u32p)]


class GmParams(C.Structure):
    _fields_ = [("box", C.c_double * 3), ("periodic", C.c_int32), ("precision", C.c_int32),
                ("r_cutoff", C.c_double), ("r_skin", C.c_double), ("r_switch", C.c_double),
                ("max_constr_iter", C.c_uint32), ("constr_tol", C.c_double), ("coulomb", C.c_int32),
                ("scale14_lj", C.c_double), ("scale14_coul", C.c_double), ("device", C.c_int32),
                ("bonded_min_image", C.c_int32)]


class GmConvergence(C.Structure):
    _fields_ = [("step", C.c_uint64), ("constraint_idx", C.c_int64), ("atom_i", C.c_int64), ("atom_j", C.c_int64),
                ("residual", C.c_double), ("max_iter", C.c_uint32)]


@dataclasses.dataclass
class SimParams:
    """The SimParams fields on the path (geodesic-core/src/params.rs:4-23) plus
    the backend's own options."""

    box_size: tuple = (1000.0, 1000.0, 1000.0)
    periodic: bool = False
    r_cutoff: float = 12.0
    r_skin: float = 14.0
    r_switch: float = 10.0
    max_constr_iter: int = 100
    constr_tol: float = 1e-10
    precision: int = PRECISION_MIXED
    coulomb: bool = False
    scale14_lj: float = 0.0
    scale14_coul: float = 0.0
    device: int = 0
    # with periodic: bonded, 1-4 and constraint differences at the nearest image
    bonded_min_image: bool = False

    def to_c(self) -> GmParams:
        return GmParams((C.c_double * 3)(*self.box_size), int(self.periodic), int(self.precision), self.r_cutoff,
                        self.r_skin, self.r_switch, int(self.max_constr_iter), self.constr_tol, int(self.coulomb),
                        self.scale14_lj, self.scale14_coul, int(self.device), int(self.bonded_min_image))


_lib = None


def library_path() -> str:
    return _build.CUDA_LIB


def lib():
    """Loads the in-tree C-ABI library; raises if it was never built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise BackendError(2, f"CUDA backend library not built: {path} (run __graft_entry__.build())")
        L = C.CDLL(path)
        P = C.POINTER
        L.gm_create.restype = C.c_void_p
        L.gm_create.argtypes = [P(GmAtoms), P(GmTopology), P(GmParams), P(C.c_int32)]
        L.gm_destroy.argtypes = [C.c_void_p]
        L.gm_build_list.argtypes = [C.c_void_p, _f64p, _f64p, _f64p]
        L.gm_compute_forces.argtypes = [C.c_void_p] + [_f64p] * 7
        L.gm_needs_rebuild.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, P(C.c_int32)]
        L.gm_geodesic_drift.argtypes = [C.c_void_p] + [_f64p] * 6 + [C.c_double, C.c_uint64, P(GmConvergence)]
        L.gm_half_kick.argtypes = [C.c_void_p] + [_f64p] * 6 + [C.c_double]
        L.gm_constrain_velocities.argtypes = [C.c_void_p] + [_f64p] * 6 + [C.c_uint64, P(GmConvergence)]
        L.gm_kinetic_energy.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, _f64p]
        L.gm_n_threads.argtypes = [C.c_void_p]
        L.gm_get_pairs.argtypes = [C.c_void_p, C.c_int64, _u32p, _u32p, P(C.c_int64)]
        # row pointers as plain addresses: a call per step stays cheap
        L.gm_steps.argtypes = [C.c_void_p] + [C.c_void_p] * 6 + [C.c_double, C.c_uint64, C.c_int64] + [
            C.c_void_p] * 3 + [_f64p, P(C.c_int64), P(GmConvergence)]
        L.gm_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_int64]
        L.gm_frames_enable.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        L.gm_frames_take.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     P(C.c_int64), P(C.c_int64)]
        L.gm_upload_state.argtypes = [C.c_void_p] + [_f64p] * 6
        L.gm_download_state.argtypes = [C.c_void_p] + [_f64p] * 6
        L.gm_run_resident.argtypes = [C.c_void_p, C.c_double, C.c_uint64, C.c_int64]
        L.gm_forces_resident.argtypes = [C.c_void_p]
        L.gm_synchronize.argtypes = [C.c_void_p, P(GmConvergence)]
        L.gm_stream.restype = C.c_void_p
        L.gm_stream.argtypes = [C.c_void_p]
        L.gm_counters.argtypes = [C.c_void_p, P(C.c_int64), C.c_int64]
        L.gm_profile.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_double, P(C.c_double)]
        L.gm_time_steps.argtypes = [C.c_void_p, C.c_double, C.c_uint64, C.c_int64, C.c_void_p, C.c_int64,
                                    P(C.c_double)]
        L.gm_build_pairs_static.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, P(GmParams), C.c_void_p,
                                            C.c_void_p, C.c_int64, P(C.c_int64), C.c_void_p]
        _f32p = P(C.c_float)
        L.gm_create_ensemble.restype = C.c_void_p
        L.gm_create_ensemble.argtypes = [C.c_int32, P(GmAtoms), P(GmTopology), P(GmParams), P(C.c_int32)]
        L.gm_ensemble_info.argtypes = [C.c_void_p, P(C.c_int64)]
        L.gm_ensemble_energies.argtypes = [C.c_void_p, _f64p, _f64p]
        L.gm_autotune.argtypes = [C.c_void_p, C.c_int32, P(C.c_int64)]
        L.gm_pair_shape.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
        L.gm_step_form.argtypes = [C.c_void_p, C.c_int32]
        L.gm_stall_next_barrier.argtypes = [C.c_void_p]
        L.gm_ws_record.argtypes = [C.c_void_p, C.c_int64, C.c_int32]
        L.gm_ws_samples.argtypes = [C.c_void_p, C.c_int64, _f32p, _f32p, P(C.c_int64)]
        L.gm_ws_train.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_double, C.c_uint64, P(C.c_double)]
        L.gm_ws_enable.argtypes = [C.c_void_p, C.c_int32]
        L.gm_ws_params.argtypes = [C.c_void_p, _f32p, _f32p, _f32p, _f32p]
        L.gm_ws_forward.argtypes = [C.c_void_p, _f32p, C.c_int64, _f32p]
        L.gm_ws_gradient.argtypes = [C.c_void_p, _f32p, _f32p, C.c_int64, _f32p, P(C.c_double)]
        L.gm_ws_last.argtypes = [C.c_void_p, _f32p, _f64p, _f64p]
        for f in ("gm_autotune", "gm_ensemble_info", "gm_ensemble_energies", "gm_ws_record", "gm_ws_samples", "gm_ws_train", "gm_ws_enable", "gm_ws_params", "gm_ws_forward",
                  "gm_ws_gradient", "gm_ws_last", "gm_build_pairs_static", "gm_destroy", "gm_build_list", "gm_compute_forces", "gm_needs_rebuild", "gm_geodesic_drift",
                  "gm_half_kick", "gm_constrain_velocities", "gm_kinetic_energy", "gm_n_threads", "gm_get_pairs",
                  "gm_steps", "gm_last_error", "gm_upload_state", "gm_download_state", "gm_run_resident",
                  "gm_forces_resident", "gm_synchronize", "gm_counters", "gm_profile", "gm_time_steps",
                  "gm_frames_enable", "gm_frames_take"):
            getattr(L, f).restype = C.c_int32
        _lib = L
    return _lib


def build_pairs_static(pos_ptr, n_atoms, excl_start_ptr, excl_ptr, params: SimParams, pair_i_ptr, pair_j_ptr,
                       max_pairs, stream=None):
    """gm_build_pairs_static: the half list of at most GM_STATIC_MAX_ATOMS
    atoms from device buffers (integer device addresses), without allocating
    device memory.  Returns the pair count; raises BackendError on failure
    (status 7 with .n_pairs set when the count exceeds max_pairs)."""
    cnt = C.c_int64()
    prm = params.to_c()
    rc = lib().gm_build_pairs_static(pos_ptr, int(n_atoms), excl_start_ptr, excl_ptr, C.byref(prm), pair_i_ptr,
                                     pair_j_ptr, int(max_pairs), C.byref(cnt), stream)
    if rc:
        err = BackendError(rc, f"gm_build_pairs_static failed with status {rc}")
        err.n_pairs = cnt.value
        raise err
    return cnt.value


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def _row_addrs(a):
    """Addresses of the three rows of a C-contiguous float64 (3, N) array."""
    assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape[0] == 3, "expect C-contiguous float64 (3, N)"
    base = a.__array_interface__["data"][0]
    step = a.strides[0]
    return base, base + step, base + 2 * step


def _rows(a):
    """Three contiguous float64 rows of a (3, N) array, with their pointers."""
    assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape[0] == 3, "expect C-contiguous float64 (3, N)"
    return _p(a[0]), _p(a[1]), _p(a[2])


class CudaBackend:
    """`ComputeBackend` for `backend = "cuda"` (geodesic-core/src/backend.rs:11-23)."""

    def __init__(self, atoms, topology, params: SimParams):
        self._create([atoms], [topology], params)

    @classmethod
    def ensemble(cls, atoms_list, topo_list, params: SimParams):
        """A batch of independent systems in one context (gm_create_ensemble):
        per-atom arrays are the systems' arrays concatenated in order."""
        self = cls.__new__(cls)
        self._create(list(atoms_list), list(topo_list), params)
        return self

    def _create(self, atoms_list, topo_list, params):
        L = lib()
        assert len(atoms_list) == len(topo_list) and atoms_list
        self._atoms, self._topo, self.params = atoms_list[0], topo_list[0], params
        self.n_sys = len(atoms_list)
        keep = []
        self._keep = keep

        def f(a):
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return _p(a)

        def u(a):
            a = np.ascontiguousarray(a, dtype=np.uint32)
            keep.append(a)
            return _p(a, C.c_uint32)

        ca = (GmAtoms * self.n_sys)()
        ct = (GmTopology * self.n_sys)()
        sizes = []
        for k, (atoms, t) in enumerate(zip(atoms_list, topo_list)):
            n = int(len(atoms.mass))
            sizes.append(n)
            el = getattr(atoms, "element", None)
            elp = None
            if el is not None:
                el = np.ascontiguousarray(el, dtype=np.uint8)
                keep.append(el)
                elp = _p(el, C.c_uint8)
            ca[k] = GmAtoms(n, f(atoms.sigma), f(atoms.epsilon), f(atoms.mass),
                            f(getattr(atoms, "charge", np.zeros(n))), elp)
            ct[k] = GmTopology(len(t.bond_i), u(t.bond_i), u(t.bond_j), f(t.bond_k), f(t.bond_r0),
                               len(t.angle_i), u(t.angle_i), u(t.angle_j), u(t.angle_k), f(t.angle_kth),
                               f(t.angle_th0), len(t.dihed_i), u(t.dihed_i), u(t.dihed_j), u(t.dihed_k),
                               u(t.dihed_l), f(t.dihed_kphi), u(t.dihed_n), f(t.dihed_delta), len(t.constr_i),
                               u(t.constr_i), u(t.constr_j), f(t.constr_dsq), len(t.excl_i), u(t.excl_i),
                               u(t.excl_j))
        self.n = int(sum(sizes))
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        st = C.c_int32()
        cp = params.to_c()
        if self.n_sys == 1:
            self._h = L.gm_create(C.byref(ca[0]), C.byref(ct[0]), C.byref(cp), C.byref(st))
        else:
            self._h = L.gm_create_ensemble(self.n_sys, ca, ct, C.byref(cp), C.byref(st))
        if not self._h:
            raise BackendError(st.value, "gm_create failed")
        self._forces = np.zeros((3, self.n))
        self._energy = 0.0
        self._steps_out = None  # reused gm_steps out-parameters
        self._addr_cache = {}   # id(array) -> (array, shape, strides, row addresses)

    def autotune(self, reps=5):
        """Pick the pair kernel's split, block size and grid by timing
        (gm_autotune); returns them."""
        out = (C.c_int64 * 3)()
        self._check(lib().gm_autotune(self._h, int(reps), out))
        return dict(split=out[0], warps_per_block=out[1], grid=out[2])

    def pair_shape(self, split, warps_per_block, grid=0):
        """Sets the pair kernel's launch shape (gm_pair_shape), e.g. a cached
        autotune() result."""
        self._check(lib().gm_pair_shape(self._h, int(split), int(warps_per_block), int(grid)))

    def step_form(self, form):
        """How resident steps are issued (gm_step_form): STEP_GRAPH, the
        kernel graph, or STEP_PERSISTENT, one persistent cooperative launch per
        step (unconstrained mixed-precision contexts).  Same bits either way."""
        self._check(lib().gm_step_form(self._h, int(form)))

    def ensemble_energies(self):
        """Per-system (potential, kinetic) energies (gm_ensemble_energies)."""
        ep = np.zeros(self.n_sys)
        ek = np.zeros(self.n_sys)
        self._check(lib().gm_ensemble_energies(self._h, _p(ep), _p(ek)))
        return ep, ek

    def frames_enable(self, frame_interval: int, capacity: int = 64):
        """Record a trajectory frame every `frame_interval` resident steps into
        a device ring of `capacity` frames (gm_frames_enable); 0 turns it off."""
        self._check(lib().gm_frames_enable(self._h, int(frame_interval), int(capacity)))
        self._frame_cap = int(capacity) if frame_interval > 0 else 0

    def frames_take(self):
        """The frames recorded since the last call (gm_frames_take): xyz
        (n, 3, N) float32, step (n,) uint64, e_pot and e_kin (n,) float64."""
        cap = getattr(self, "_frame_cap", 0)
        xyz = np.zeros((cap, 3, self.n), dtype=np.float32)
        steps = np.zeros(cap, dtype=np.uint64)
        ep = np.zeros(cap)
        ek = np.zeros(cap)
        n, lost = C.c_int64(), C.c_int64()
        self._check(lib().gm_frames_take(self._h, cap, xyz.ctypes.data, steps.ctypes.data, ep.ctypes.data,
                                         ek.ctypes.data, C.byref(n), C.byref(lost)))
        if lost.value:
            raise BackendError(GM_ERR_INVALID_ARGUMENT, f"{lost.value} trajectory frames lost on a full ring")
        k = n.value
        return dict(xyz=xyz[:k], step=steps[:k], e_pot=ep[:k], e_kin=ek[:k])

    def resident_energies(self):
        """(potential, kinetic) energy of the resident state, summed over the
        systems of a batch."""
        ep, ek = self.ensemble_energies()
        return float(ep.sum()), float(ek.sum())

    def close(self):
        if getattr(self, "_h", None):
            lib().gm_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, rc, conv=None):
        if rc == GM_OK:
            return
        buf = C.create_string_buffer(1024)
        lib().gm_last_error(self._h, buf, 1024)
        msg = buf.value.decode(errors="replace")
        if rc == 5 and conv is not None:
            raise ConvergenceError(rc, msg, conv)
        if rc == 6:
            raise NumericalError(rc, msg)
        raise BackendError(rc, msg)

    # ---------------------------------------------------------- trait
    def build_neighbor_list(self, pos: np.ndarray) -> None:
        """backend.rs:14: wraps `pos` in place when periodic."""
        self._check(lib().gm_build_list(self._h, *_rows(pos)))

    def compute_forces(self, pos: np.ndarray) -> np.ndarray:
        """backend.rs:15: forces (3, N) at `pos`; energy in potential_energy()."""
        e = C.c_double()
        rc = lib().gm_compute_forces(self._h, *_rows(np.ascontiguousarray(pos)), *_rows(self._forces), C.byref(e))
        self._energy = e.value
        self._check(rc)
        return self._forces

    def geodesic_drift(self, pos: np.ndarray, vel: np.ndarray, dt: float, step: int = 0) -> None:
        """backend.rs:16: drift + SHAKE + velocity resync, in place."""
        conv = GmConvergence()
        self._check(lib().gm_geodesic_drift(self._h, *_rows(pos), *_rows(vel), dt, step, C.byref(conv)), conv)

    def reduce_forces(self) -> np.ndarray:
        """backend.rs:17"""
        return self._forces.copy()

    def potential_energy(self) -> float:
        """backend.rs:18"""
        return self._energy

    def atoms(self):
        return self._atoms

    def topology(self):
        return self._topo

    def needs_rebuild(self, pos: np.ndarray) -> bool:
        """backend.rs:21"""
        r = C.c_int32()
        self._check(lib().gm_needs_rebuild(self._h, *_rows(np.ascontiguousarray(pos)), C.byref(r)))
        return bool(r.value)

    def n_threads(self) -> int:
        return int(lib().gm_n_threads(self._h))

    # ------------------------------------------ engine free functions
    def half_kick(self, vel: np.ndarray, force: np.ndarray, dt_half: float) -> None:
        """integrator::half_kick (integrator.rs:14-21)."""
        self._check(lib().gm_half_kick(self._h, *_rows(vel), *_rows(np.ascontiguousarray(force)), dt_half))

    def constrain_velocities(self, pos: np.ndarray, vel: np.ndarray, step: int = 0) -> None:
        """constraint::constrain_velocities (constraint.rs:170-259)."""
        conv = GmConvergence()
        self._check(lib().gm_constrain_velocities(self._h, *_rows(np.ascontiguousarray(pos)), *_rows(vel), step,
                                                  C.byref(conv)), conv)

    def kinetic_energy(self, vel: np.ndarray) -> float:
        """lib.rs:68-77"""
        ke = C.c_double()
        self._check(lib().gm_kinetic_energy(self._h, *_rows(np.ascontiguousarray(vel)), C.byref(ke)))
        return ke.value

    # ---------------------------------------------------- extras
    def pairs(self):
        """The current list as the reference's NeighborList pair_i/pair_j."""
        L = lib()
        cnt = C.c_int64()
        self._check(L.gm_get_pairs(self._h, 0, None, None, C.byref(cnt)))
        pi = np.zeros(max(cnt.value, 1), np.uint32)
        pj = np.zeros(max(cnt.value, 1), np.uint32)
        self._check(L.gm_get_pairs(self._h, cnt.value, _p(pi, C.c_uint32), _p(pj, C.c_uint32), C.byref(cnt)))
        return pi[:cnt.value], pj[:cnt.value]

    def steps(self, pos, vel, dt, n_steps, first_step=0, want_forces=False):
        """Device-resident BAB + RATTLE steps (lib.rs:292-323), state in place.
        Returns (potential energy, list rebuilds, forces or None)."""
        out = self._steps_out
        if out is None:
            e, nr, conv = C.c_double(), C.c_int64(), GmConvergence()
            out = self._steps_out = (e, nr, conv, C.byref(e), C.byref(nr), C.byref(conv))
        e, nr, conv, e_ref, nr_ref, conv_ref = out
        f = np.zeros((3, self.n)) if want_forces else None
        fr = _row_addrs(f) if want_forces else (None, None, None)
        rc = lib().gm_steps(self._h, *self._addrs(pos), *self._addrs(vel), dt, first_step, n_steps, *fr, e_ref,
                            nr_ref, conv_ref)
        if rc != GM_OK:
            self._check(rc, GmConvergence.from_buffer_copy(conv))
        self._energy = e.value
        return e.value, nr.value, f

    def stall_next_barrier(self):
        """gm_stall_next_barrier: the next persistent call's grid barrier
        waits out its poll limit and the call fails (error-path test)."""
        self._check(lib().gm_stall_next_barrier(self._h))

    def _addrs(self, a):
        """Row addresses of a (3, N) float64 array, remembered for the arrays
        a step loop passes call after call (the cache holds a reference, so
        numpy cannot move their data)."""
        hit = self._addr_cache.get(id(a))
        if hit is not None and hit[0] is a and hit[1] == a.shape and hit[2] == a.strides:
            return hit[3]
        addrs = _row_addrs(a)
        if len(self._addr_cache) >= 8:
            self._addr_cache.clear()
        self._addr_cache[id(a)] = (a, a.shape, a.strides, addrs)
        return addrs

    def upload_state(self, pos, vel):
        self._check(lib().gm_upload_state(self._h, *_rows(np.ascontiguousarray(pos)), *_rows(np.ascontiguousarray(vel))))

    def download_state(self, pos, vel):
        self._check(lib().gm_download_state(self._h, *_rows(pos), *_rows(vel)))

    def run_resident(self, dt, n_steps, first_step=0):
        self._check(lib().gm_run_resident(self._h, dt, first_step, n_steps))

    def forces_resident(self):
        self._check(lib().gm_forces_resident(self._h))

    def synchronize(self):
        conv = GmConvergence()
        self._check(lib().gm_synchronize(self._h, C.byref(conv)), conv)

    def profile(self, which: str, n_iter: int = 20, dt: float = 0.002) -> float:
        """Average device milliseconds of one launch (CUDA events)."""
        code = {"pair": 0, "bonded": 1, "rebuild": 2, "step": 3, "pack": 4, "forces": 5, "pair14": 6, "build": 7}[which]
        ms = C.c_double()
        self._check(lib().gm_profile(self._h, code, n_iter, dt, C.byref(ms)))
        return ms.value

    def time_steps(self, dt: float, n_steps: int, first_step: int = 0, flush_ptr: int = 0,
                   flush_bytes: int = 0) -> float:
        """Sum of per-step device milliseconds over n_steps resident steps
        (L2 flushed between steps when a flush buffer is given)."""
        ms = C.c_double()
        self._check(lib().gm_time_steps(self._h, dt, first_step, n_steps, C.c_void_p(flush_ptr or None),
                                        flush_bytes, C.byref(ms)))
        return ms.value

    def stream(self) -> int:
        return int(lib().gm_stream(self._h) or 0)

    def counters(self) -> dict:
        out = (C.c_int64 * 12)()
        self._check(lib().gm_counters(self._h, out, 12))
        return dict(pairs=out[0], rebuilds=out[1], cap=out[2], launches=out[3], shake_iters=out[4],
                    rattle_iters=out[5], launches_per_step=out[6], split=out[7], constrained_steps=out[8],
                    shake_iter_sum=out[9], rattle_iter_sum=out[10], ws_records=out[11])

    # ------------------------------------------- constraint warm start
    WS_NPAR, WS_NNORM = 5057, 26

    def ws_record(self, cap_steps, stride=1):
        """Record (features, multiplier target) of every stride-th resident solve."""
        self._check(lib().gm_ws_record(self._h, int(cap_steps), int(stride)))

    def ws_samples(self):
        n = C.c_int64()
        self._check(lib().gm_ws_samples(self._h, 0, None, None, C.byref(n)))
        f = np.zeros((max(n.value, 1), 12), np.float32)
        t = np.zeros(max(n.value, 1), np.float32)
        self._check(lib().gm_ws_samples(self._h, n.value, _p(f, C.c_float), _p(t, C.c_float), C.byref(n)))
        return f[:n.value], t[:n.value]

    def ws_train(self, iters, blocks=64, lr=3e-3, seed=1):
        """Train the warm-start network on the recorded samples; returns the last batch loss."""
        loss = C.c_double()
        self._check(lib().gm_ws_train(self._h, int(iters), int(blocks), float(lr), int(seed), C.byref(loss)))
        return loss.value

    def ws_enable(self, on=True):
        self._check(lib().gm_ws_enable(self._h, 1 if on else 0))

    def ws_params(self, params=None, norm=None):
        """Sets the parameters/norm when given; returns the current ones."""
        sp = None if params is None else np.ascontiguousarray(params, np.float32)
        sn = None if norm is None else np.ascontiguousarray(norm, np.float32)
        if sp is not None or sn is not None:
            self._check(lib().gm_ws_params(self._h, None, None, None if sp is None else _p(sp, C.c_float),
                                           None if sn is None else _p(sn, C.c_float)))
        gp = np.zeros(self.WS_NPAR, np.float32)
        gn = np.zeros(self.WS_NNORM, np.float32)
        self._check(lib().gm_ws_params(self._h, _p(gp, C.c_float), _p(gn, C.c_float), None, None))
        return gp, gn

    def ws_forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(len(x), np.float32)
        self._check(lib().gm_ws_forward(self._h, _p(x, C.c_float), len(x), _p(y, C.c_float)))
        return y

    def ws_gradient(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.WS_NPAR, np.float32)
        loss = C.c_double()
        self._check(lib().gm_ws_gradient(self._h, _p(x, C.c_float), _p(t, C.c_float), len(x), _p(g, C.c_float),
                                         C.byref(loss)))
        return g, loss.value

    def ws_last(self, n_constr):
        f = np.zeros((max(n_constr, 1), 12), np.float32)
        l0 = np.zeros(max(n_constr, 1))
        ls = np.zeros(max(n_constr, 1))
        self._check(lib().gm_ws_last(self._h, _p(f, C.c_float), _p(l0), _p(ls)))
        return f[:n_constr], l0[:n_constr], ls[:n_constr]
