"""A CPU stand-in for the resident-state methods of `CudaBackend` that
`geodesic_cuda.run` calls, built on the oracle's restatement of the
reference's step (oracle/oracle.py).  It gives the run loop's orchestration
(initial velocity projection, frame 0, frame numbering and draining, batch
offsets, drift checks, summaries) a CPU test: each resident step is the body
of lib.rs:292-323 on the oracle's calls, in the order `or_run` uses, so a
run through this stand-in writes the frames `oracle.run` returns.

Only the checker uses it; the product path always builds a `CudaBackend`."""
import numpy as np

import oracle


class OracleResident:
    def __init__(self, atoms_list, topo_list, params):
        self.p = oracle.make_params(box=tuple(params.box_size), periodic=params.periodic, r_cutoff=params.r_cutoff,
                                    r_skin=params.r_skin, r_switch=params.r_switch,
                                    max_constr_iter=params.max_constr_iter, constr_tol=params.constr_tol, n_threads=1,
                                    bonded_min_image=params.bonded_min_image)
        self.box = tuple(params.box_size) if params.periodic and params.bonded_min_image else None
        self.max_iter, self.tol = params.max_constr_iter, params.constr_tol
        self.systems = [(a, t, oracle.CpuBackend(a, t, self.p)) for a, t in zip(atoms_list, topo_list)]
        sizes = [a.n for a in atoms_list]
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.n, self.n_sys = int(self.offsets[-1]), len(sizes)
        self.pos = self.vel = self.force = None
        self.built = False  # a list build on the host arrays that the resident forces reuse
        self.e_pot = np.zeros(self.n_sys)
        self.fi, self.cap, self.ring, self.lost = 0, 0, [], 0
        self.calls = []
        self.closed = False

    def _sl(self, k):
        return slice(int(self.offsets[k]), int(self.offsets[k + 1]))

    # ------------------------------------------------------------ state
    def build_neighbor_list(self, pos):
        """The trait's list build on host arrays (wraps a periodic system in
        place); the next forces_resident reuses these lists."""
        self.calls.append("build_neighbor_list")
        for k, (_, _, b) in enumerate(self.systems):
            sl = self._sl(k)
            p = np.ascontiguousarray(pos[:, sl])
            b.build_neighbor_list(p)
            pos[:, sl] = p
        self.built = True

    def constrain_velocities(self, pos, vel, step=0):
        self.calls.append("constrain_velocities")
        for k, (a, t, _) in enumerate(self.systems):
            sl = self._sl(k)
            p, v = np.ascontiguousarray(pos[:, sl]), np.ascontiguousarray(vel[:, sl])
            oracle.constrain_velocities(t, a, p, v, self.max_iter, self.tol, step, box=self.box)
            vel[:, sl] = v

    def upload_state(self, pos, vel):
        self.calls.append("upload_state")
        self.pos = [np.ascontiguousarray(pos[:, self._sl(k)]).copy() for k in range(self.n_sys)]
        self.vel = [np.ascontiguousarray(vel[:, self._sl(k)]).copy() for k in range(self.n_sys)]
        self.force = None

    def download_state(self, pos, vel):
        self.calls.append("download_state")
        for k in range(self.n_sys):
            pos[:, self._sl(k)] = self.pos[k]
            vel[:, self._sl(k)] = self.vel[k]

    def forces_resident(self):
        self.calls.append("forces_resident")
        self.force = []
        for k, (_, _, b) in enumerate(self.systems):
            if not self.built:
                b.build_neighbor_list(self.pos[k])
            self.force.append(b.compute_forces(self.pos[k]))
            self.e_pot[k] = b.potential_energy
        self.built = False

    def _kinetic(self):
        return np.array([oracle.kinetic_energy(self.vel[k], a.mass) for k, (a, _, _) in enumerate(self.systems)])

    def ensemble_energies(self):
        assert self.force is not None, "no forces at the resident positions"
        return self.e_pot.copy(), self._kinetic()

    def resident_energies(self):
        ep, ek = self.ensemble_energies()
        return float(ep.sum()), float(ek.sum())

    # ------------------------------------------------------------ steps
    def run_resident(self, dt, n_steps, first_step=0):
        self.calls.append(("run_resident", n_steps, first_step))
        assert self.force is not None
        for step in range(first_step, first_step + n_steps):
            for k, (a, t, b) in enumerate(self.systems):
                p, v = self.pos[k], self.vel[k]
                oracle.half_kick(v, self.force[k], a.mass, dt / 2.0)
                b.geodesic_drift(p, v, dt, step)
                if b.needs_rebuild(p):
                    b.build_neighbor_list(p)
                self.force[k] = b.compute_forces(p)
                self.e_pot[k] = b.potential_energy
                oracle.half_kick(v, self.force[k], a.mass, dt / 2.0)
                oracle.constrain_velocities(t, a, p, v, self.max_iter, self.tol, step, box=self.box)
            if self.fi and (step + 1) % self.fi == 0:
                if len(self.ring) == self.cap:
                    self.lost += 1
                else:
                    xyz = np.concatenate(self.pos, axis=1).astype(np.float32)
                    self.ring.append((step + 1, xyz, float(self.e_pot.sum()), float(self._kinetic().sum())))

    def frames_enable(self, frame_interval, capacity=64):
        self.calls.append(("frames_enable", frame_interval, capacity))
        self.fi, self.cap, self.ring, self.lost = int(frame_interval), int(capacity), [], 0

    def frames_take(self):
        assert not self.lost, "frames lost on a full ring"
        fr = self.ring
        self.ring = []
        return dict(xyz=np.array([f[1] for f in fr], np.float32).reshape(len(fr), 3, self.n),
                    step=np.array([f[0] for f in fr], np.uint64), e_pot=np.array([f[2] for f in fr]),
                    e_kin=np.array([f[3] for f in fr]))

    def close(self):
        self.closed = True


def make(atoms_list, topo_list, params):
    """`make_backend` for `geodesic_cuda.run`."""
    return OracleResident(atoms_list, topo_list, params)
