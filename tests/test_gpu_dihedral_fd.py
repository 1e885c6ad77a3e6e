"""Device dihedral forces against finite differences of the FP64 energy
(needs a GPU).

The reference's README (README.md:53-55) calls its dihedral forces incorrect
for general geometry, while its bonded code and ROADMAP say the formula was
fixed and checked by finite differences on two geometries
(geodesic-engine/tests/bonded_gradient.rs:118-165).  Here the device's
dihedral forces, in both precisions, are compared with central differences
(eps = 1e-6 A) of the oracle's FP64 dihedral energy (force/bonded.rs:112-164
restated) on 200 seeded quads: general geometries, torsions within 1e-3 rad
of 0 and of pi, and arms within ~0.6 degrees of collinear.  The bound is the
reference harness's: |F - F_fd| / (|F_fd| + 1) < 1e-4
(bonded_gradient.rs:32-68).
"""
import numpy as np
import pytest

import oracle
from geodesic_cuda import amber, backend

pytestmark = pytest.mark.gpu

N_QUADS = 200
EPS = 1e-6


def place(l1, l2, l3, th1, th2, phi):
    """Four points with bond lengths l1..l3, bond angles th1 (at atom 2) and
    th2 (at atom 3) and torsion phi (natural extension of reference frame)."""
    p0 = np.zeros(3)
    p1 = np.array([l1, 0.0, 0.0])
    p2 = p1 + l2 * np.array([-np.cos(th1), np.sin(th1), 0.0])
    b1, b2 = p1 - p0, p2 - p1
    e2 = b2 / np.linalg.norm(b2)
    nrm = np.cross(b1, b2)
    nrm /= np.linalg.norm(nrm)
    m = np.cross(nrm, e2)
    d = np.array([-np.cos(th2), np.sin(th2) * np.cos(phi), np.sin(th2) * np.sin(phi)])
    p3 = p2 + l3 * (d[0] * e2 + d[1] * m + d[2] * nrm)
    return np.stack([p0, p1, p2, p3])


def quads(seed=2024):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(N_QUADS):
        l1, l2, l3 = rng.uniform(1.0, 2.0, 3)
        th1, th2 = rng.uniform(np.deg2rad(60), np.deg2rad(150), 2)
        phi = rng.uniform(-np.pi, np.pi)
        kind = q % 5
        if kind == 1:
            phi = rng.uniform(-1e-3, 1e-3)                  # near cis
        elif kind == 2:
            phi = np.pi + rng.uniform(-1e-3, 1e-3)          # near trans
        elif kind == 3:
            th1 = np.pi - rng.uniform(0.005, 0.01)          # first arm nearly collinear
        elif kind == 4:
            th2 = np.pi - rng.uniform(0.005, 0.01)          # last arm nearly collinear
        pts = place(l1, l2, l3, th1, th2, phi)
        # a random rigid rotation and an offset that keeps quads apart
        a = rng.normal(size=(3, 3))
        rot, _ = np.linalg.qr(a)
        pts = pts @ rot.T + np.array([60.0 * (q % 15), 60.0 * (q // 15), 0.0])
        out.append(pts)
    return np.concatenate(out, axis=0)  # (4 N_QUADS, 3)


def system():
    pts = quads()
    n = len(pts)
    rng = np.random.default_rng(7)
    t = amber.BondedTopology.empty()
    idx = np.arange(N_QUADS, dtype=np.uint32) * 4
    t.dihed_i, t.dihed_j, t.dihed_k, t.dihed_l = idx, idx + 1, idx + 2, idx + 3
    t.dihed_kphi = rng.uniform(0.5, 3.5, N_QUADS)
    t.dihed_n = rng.integers(1, 5, N_QUADS).astype(np.uint32)
    t.dihed_delta = rng.uniform(0.0, 2 * np.pi, N_QUADS)
    atoms = amber.AtomData(np.zeros(n), np.zeros(n), np.ones(n), np.zeros(n), np.full(n, 5, np.uint8),
                           np.zeros(n, np.uint32), ["C   "] * n)
    return atoms, t, np.ascontiguousarray(pts.T)


def fd_forces(pos, topo):
    """-dV/dx by central differences of the oracle's FP64 dihedral energy."""
    f = np.zeros_like(pos)
    for d in range(3):
        for i in range(pos.shape[1]):
            p = pos.copy()
            p[d, i] += EPS
            vp, _ = oracle.bonded_forces("dihedral", p, topo)
            p[d, i] -= 2 * EPS
            vm, _ = oracle.bonded_forces("dihedral", p, topo)
            f[d, i] = -(vp - vm) / (2 * EPS)
    return f


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_dihedral_forces_match_finite_differences(precision):
    atoms, topo, pos = system()
    be = backend.CudaBackend(atoms, topo, backend.SimParams(precision=precision, box_size=(10000.0,) * 3,
                                                            periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0))
    p = pos.copy()
    be.build_neighbor_list(p)
    f = be.compute_forces(p).copy()
    be.close()
    f_fd = fd_forces(pos, topo)
    rel = np.abs(f - f_fd) / (np.abs(f_fd) + 1.0)
    assert rel.max() < 1e-4, (rel.max(), np.unravel_index(rel.argmax(), rel.shape))
    # and the oracle's analytic forces (the reference formula) to FP64 round-off
    _, f_or = oracle.bonded_forces("dihedral", pos.copy(), topo)
    assert np.all(np.abs(f - f_or) <= 1e-10 * np.maximum(np.abs(f_or), 1.0))
