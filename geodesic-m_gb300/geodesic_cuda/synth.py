"""Seeded synthetic systems (jittered-lattice serpentine chains), see
`synth/gmsynth.c` for the recipe.  Returns the same AtomData /
BondedTopology / State triple the AMBER readers produce."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build, amber

_lib = None


class _Req(C.Structure):
    _fields_ = [("n_atoms", C.c_int64), ("seed", C.c_uint64), ("h_fraction", C.c_double),
                ("temperature", C.c_double), ("relax_iters", C.c_int32), ("n_threads", C.c_int32)]


class _Sizes(C.Structure):
    _fields_ = [("n_atoms", C.c_int64), ("n_bonds", C.c_int64), ("n_angles", C.c_int64),
                ("n_diheds", C.c_int64), ("n_excl", C.c_int64), ("n_types", C.c_int64)]


_P = lambda t: C.POINTER(t)  # noqa: E731


class _Out(C.Structure):
    _fields_ = [("pos", _P(C.c_double)), ("vel", _P(C.c_double)), ("sigma", _P(C.c_double)),
                ("epsilon", _P(C.c_double)), ("mass", _P(C.c_double)), ("charge", _P(C.c_double)),
                ("element", _P(C.c_uint8)), ("type", _P(C.c_int32)),
                ("bond_i", _P(C.c_uint32)), ("bond_j", _P(C.c_uint32)), ("bond_k", _P(C.c_double)),
                ("bond_r0", _P(C.c_double)),
                ("angle_i", _P(C.c_uint32)), ("angle_j", _P(C.c_uint32)), ("angle_k", _P(C.c_uint32)),
                ("angle_kth", _P(C.c_double)), ("angle_th0", _P(C.c_double)),
                ("dihed_i", _P(C.c_uint32)), ("dihed_j", _P(C.c_uint32)), ("dihed_k", _P(C.c_uint32)),
                ("dihed_l", _P(C.c_uint32)), ("dihed_kphi", _P(C.c_double)), ("dihed_n", _P(C.c_uint32)),
                ("dihed_delta", _P(C.c_double)), ("excl_i", _P(C.c_uint32)), ("excl_j", _P(C.c_uint32)),
                ("max_force_before", C.c_double), ("max_force_after", C.c_double)]


def _get():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build_synth())
        L.gs_sizes_for.argtypes = [_P(_Req), _P(_Sizes)]
        L.gs_generate.argtypes = [_P(_Req), _P(_Sizes), _P(_Out)]
        _lib = L
    return _lib


def generate(n_atoms: int, seed: int, h_fraction: float = 0.0, temperature: float = 300.0,
             relax_iters: int = 300, n_threads: int = 0):
    """Returns (AtomData, BondedTopology, State, info dict)."""
    L = _get()
    nt = n_threads or min(os.cpu_count() or 1, 32)
    req = _Req(n_atoms, seed & 0xFFFFFFFFFFFFFFFF, h_fraction, temperature, relax_iters, nt)
    sz = _Sizes()
    L.gs_sizes_for(C.byref(req), C.byref(sz))
    n = sz.n_atoms
    arrs = {}

    def f(name, shape):
        arrs[name] = np.zeros(shape, np.float64)
        return arrs[name].ctypes.data_as(_P(C.c_double))

    def u(name, size, dt=np.uint32, ct=C.c_uint32):
        arrs[name] = np.zeros(max(size, 0), dt)
        return arrs[name].ctypes.data_as(_P(ct))

    out = _Out(f("pos", (3, n)), f("vel", (3, n)), f("sigma", n), f("epsilon", n), f("mass", n), f("charge", n),
               u("element", n, np.uint8, C.c_uint8), u("type", n, np.int32, C.c_int32),
               u("bond_i", sz.n_bonds), u("bond_j", sz.n_bonds), f("bond_k", sz.n_bonds), f("bond_r0", sz.n_bonds),
               u("angle_i", sz.n_angles), u("angle_j", sz.n_angles), u("angle_k", sz.n_angles),
               f("angle_kth", sz.n_angles), f("angle_th0", sz.n_angles),
               u("dihed_i", sz.n_diheds), u("dihed_j", sz.n_diheds), u("dihed_k", sz.n_diheds),
               u("dihed_l", sz.n_diheds), f("dihed_kphi", sz.n_diheds), u("dihed_n", sz.n_diheds),
               f("dihed_delta", sz.n_diheds), u("excl_i", sz.n_excl), u("excl_j", sz.n_excl), 0.0, 0.0)
    rc = L.gs_generate(C.byref(req), C.byref(sz), C.byref(out))
    if rc != 0:
        raise RuntimeError("synthetic generator: inconsistent sizes")
    a = arrs
    atoms = amber.AtomData(a["sigma"], a["epsilon"], a["mass"], a["charge"], a["element"],
                           np.zeros(n, np.uint32), ["H   " if e == 0 else "C   " for e in a["element"]])
    topo = amber.BondedTopology(
        a["bond_i"], a["bond_j"], a["bond_k"], a["bond_r0"], a["angle_i"], a["angle_j"], a["angle_k"],
        a["angle_kth"], a["angle_th0"], a["dihed_i"], a["dihed_j"], a["dihed_k"], a["dihed_l"], a["dihed_kphi"],
        a["dihed_n"], a["dihed_delta"], np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0),
        a["excl_i"], a["excl_j"])
    state = amber.State(pos=a["pos"], vel=a["vel"])
    info = dict(n_atoms=n, seed=seed, h_fraction=h_fraction, temperature=temperature, relax_iters=relax_iters,
                max_force_before=out.max_force_before, max_force_after=out.max_force_after,
                n_types=sz.n_types, type=a["type"], edge=float(np.ceil(round(n ** (1 / 3), 9)) * 2.15))
    return atoms, topo, state, info
