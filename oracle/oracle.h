/*
 * oracle.h — CPU restatement of the GEODESIC-M reference engine (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * backend: only tests, the smoke check and the CPU-baseline leg of the bench
 * may load it.  The product path never calls into it.
 *
 * Every function restates one reference function with the same operation
 * order, so that results are bit-identical to the reference on the same
 * platform libm (the file:line of the restated code is given beside each
 * declaration; paths are relative to the reference repository root).  Build
 * with -ffp-contract=off: the reference (Rust) never fuses a*b+c.
 *
 * Terms marked "beyond reference" (Coulomb, scaled 1-4 pairs) have no
 * reference counterpart; they use the formulas stated at their declaration.
 */
#ifndef GEODESIC_ORACLE_H
#define GEODESIC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* AtomData (geodesic-core/src/atoms.rs:3-12). element: 0 = H (only H matters). */
typedef struct {
    int64_t n;
    const double *sigma, *epsilon, *mass, *charge;
    const uint8_t *element;
} or_atoms;

/* BondedTopology (geodesic-core/src/topology.rs:4-37), SoA, uint32 indices. */
typedef struct {
    int64_t n_bonds;  const uint32_t *bond_i, *bond_j; const double *bond_k, *bond_r0;
    int64_t n_angles; const uint32_t *angle_i, *angle_j, *angle_k; const double *angle_kth, *angle_th0;
    int64_t n_diheds; const uint32_t *dihed_i, *dihed_j, *dihed_k, *dihed_l;
    const double *dihed_kphi; const uint32_t *dihed_n; const double *dihed_delta;
    int64_t n_constr; const uint32_t *constr_i, *constr_j; const double *constr_dsq;
    int64_t n_excl;   const uint32_t *excl_i, *excl_j;
} or_topology;

/* SimParams (geodesic-core/src/params.rs:4-23), the fields the path reads. */
typedef struct {
    double box[3];
    int32_t periodic;
    int32_t n_threads;        /* 0 = all host cores (cpu_backend.rs:52-57) */
    double r_cutoff, r_skin, r_switch;
    uint32_t max_constr_iter;
    double constr_tol;
    /* beyond reference: Coulomb and scaled 1-4 pairs (0 = off = reference) */
    int32_t coulomb;
    double scale14_lj, scale14_coul;
    /* beyond reference: with periodic, bonded, 1-4 and constraint
     * displacements go to the nearest image (0 = off = reference) */
    int32_t bonded_min_image;
} or_params;

/* ConvergenceError::ConstraintSolver (geodesic-core/src/error.rs:50-63). */
typedef struct {
    uint64_t step;
    int64_t constraint_idx, atom_i, atom_j;
    double residual;
    uint32_t max_iter;
} or_convergence_error;

/* neighbor.rs:74-76 / :86-88 */
double or_min_image(double d, double box_len);
double or_wrap_coord(double x, double box_len);

/* neighbor.rs:8-55.  Wraps positions in place when periodic, then the O(N^2)
 * half list (i<j, r2 <= r_skin^2 after min-image, exclusions removed) in
 * (i, then j) order.  Returns the pair count; stores at most `cap` pairs. */
int64_t or_neighbor_build(int64_t n, double *px, double *py, double *pz, const or_params *p,
                          const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j);

/* Same pair set and order as or_neighbor_build (identical FP64 test), found
 * through a cell grid instead of the double loop.  Checker convenience for
 * large N; it is validated against or_neighbor_build in the tests. */
int64_t or_neighbor_build_cells(int64_t n, double *px, double *py, double *pz, const or_params *p,
                                const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j);
/* The pairs of already wrapped positions (no wrap): the fill call after a
 * counting or_neighbor_build / or_neighbor_build_cells (cells != 0). */
int64_t or_neighbor_pairs(int64_t n, const double *px, const double *py, const double *pz, const or_params *p,
                          const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j, int32_t cells);

/* neighbor.rs:60-72 */
int32_t or_needs_rebuild(int64_t n, const double *px, const double *py, const double *pz,
                         const double *rx, const double *ry, const double *rz,
                         double r_skin, double r_cutoff);

/* force/nonbonded.rs:20-82: accumulates into f*, returns the LJ energy. */
double or_pair_forces(const double *px, const double *py, const double *pz, const or_atoms *a,
                      const uint32_t *pair_i, const uint32_t *pair_j, int64_t n_pairs,
                      double r_cutoff, double r_switch, const double box[3],
                      double *fx, double *fy, double *fz);

/* beyond reference: Coulomb q_i q_j 332.0522173 / r times the same quintic
 * switch S(r) as the LJ term, over the same listed pairs (coulomb != 0). */
double or_coulomb_forces(const double *px, const double *py, const double *pz, const or_atoms *a,
                         const uint32_t *pair_i, const uint32_t *pair_j, int64_t n_pairs,
                         double r_cutoff, double r_switch, const double box[3],
                         double *fx, double *fy, double *fz);

/* beyond reference: scaled 1-4 pairs (i, l of each dihedral, deduplicated,
 * minus pairs that are also 1-2/1-3) get scale14_lj * LJ + scale14_coul *
 * Coulomb, unswitched and without cutoff (AMBER convention). */
int64_t or_pairs14(const or_topology *t, int64_t n_atoms, int64_t cap, uint32_t *p14_i, uint32_t *p14_j);
double or_pair14_forces(const double *px, const double *py, const double *pz, const or_atoms *a,
                        const uint32_t *p14_i, const uint32_t *p14_j, int64_t n14,
                        double scale_lj, double scale_coul, int32_t coulomb,
                        double *fx, double *fy, double *fz);

/* force/bonded.rs:5-40, :44-102, :112-164 */
double or_bond_forces(const double *px, const double *py, const double *pz, const or_topology *t,
                      double *fx, double *fy, double *fz);
double or_angle_forces(const double *px, const double *py, const double *pz, const or_topology *t,
                       double *fx, double *fy, double *fz);
double or_dihedral_forces(const double *px, const double *py, const double *pz, const or_topology *t,
                          double *fx, double *fy, double *fz);

/* constraint.rs:62-152 / :170-259.  Return iterations (>= 0) or -1 with *err set. */
int64_t or_constraint_solve(const or_topology *t, const or_atoms *a,
                            const double *rx, const double *ry, const double *rz,
                            double *px, double *py, double *pz,
                            uint32_t max_iter, double tol, uint64_t step, or_convergence_error *err);
int64_t or_constrain_velocities(const or_topology *t, const or_atoms *a,
                                const double *px, const double *py, const double *pz,
                                double *vx, double *vy, double *vz,
                                uint32_t max_iter, double tol, uint64_t step, or_convergence_error *err);

/* As or_constraint_solve, applying an initial displacement from predicted
 * multipliers lam0 (same update formula as one Jacobi sweep) before the
 * unchanged loop; lam_out (nullable) receives the summed multipliers
 * sum_iter lambda per constraint.  With lam0 == NULL it equals
 * or_constraint_solve.  Beyond reference (warm start). */
int64_t or_constraint_solve_ws(const or_topology *t, const or_atoms *a,
                               const double *rx, const double *ry, const double *rz,
                               double *px, double *py, double *pz,
                               uint32_t max_iter, double tol, uint64_t step,
                               const double *lam0, double *lam_out, or_convergence_error *err);

/* Beyond reference: the same functions with the displacement between the two
 * atoms of a bond, angle arm, dihedral bond vector, 1-4 pair or constraint
 * taken to the nearest image of box mi_box (or_min_image per component);
 * mi_box == NULL is the function above, bit for bit.  The reference keeps
 * these differences raw (memory.md:140-144); CpuBackend and or_run pass the
 * box when params.periodic && params.bonded_min_image. */
double or_pair14_forces_box(const double *px, const double *py, const double *pz, const or_atoms *a,
                            const uint32_t *p14_i, const uint32_t *p14_j, int64_t n14,
                            double scale_lj, double scale_coul, int32_t coulomb, const double *mi_box,
                            double *fx, double *fy, double *fz);
double or_bond_forces_box(const double *px, const double *py, const double *pz, const or_topology *t,
                          const double *mi_box, double *fx, double *fy, double *fz);
double or_angle_forces_box(const double *px, const double *py, const double *pz, const or_topology *t,
                           const double *mi_box, double *fx, double *fy, double *fz);
double or_dihedral_forces_box(const double *px, const double *py, const double *pz, const or_topology *t,
                              const double *mi_box, double *fx, double *fy, double *fz);
int64_t or_constraint_solve_box(const or_topology *t, const or_atoms *a,
                                const double *rx, const double *ry, const double *rz,
                                double *px, double *py, double *pz,
                                uint32_t max_iter, double tol, uint64_t step,
                                const double *lam0, double *lam_out, const double *mi_box,
                                or_convergence_error *err);
int64_t or_constrain_velocities_box(const or_topology *t, const or_atoms *a,
                                    const double *px, const double *py, const double *pz,
                                    double *vx, double *vy, double *vz,
                                    uint32_t max_iter, double tol, uint64_t step, const double *mi_box,
                                    or_convergence_error *err);
int64_t or_drift_and_constrain_box(int64_t n, double *px, double *py, double *pz,
                                   double *vx, double *vy, double *vz, const or_topology *t, const or_atoms *a,
                                   double dt, uint32_t max_iter, double tol, uint64_t step, const double *mi_box,
                                   or_convergence_error *err);

/* integrator.rs:14-21 and :32-71 */
void or_half_kick(int64_t n, double *vx, double *vy, double *vz,
                  const double *fx, const double *fy, const double *fz, const double *mass, double dt_half);
int64_t or_drift_and_constrain(int64_t n, double *px, double *py, double *pz,
                               double *vx, double *vy, double *vz, const or_topology *t, const or_atoms *a,
                               double dt, uint32_t max_iter, double tol, uint64_t step,
                               or_convergence_error *err);

/* geodesic/src/lib.rs:68-77 */
double or_kinetic_energy(int64_t n, const double *vx, const double *vy, const double *vz, const double *mass);

/* CpuBackend (geodesic-engine/src/cpu_backend.rs:25-219) */
typedef struct or_backend or_backend;
or_backend *or_backend_new(const or_atoms *a, const or_topology *t, const or_params *p);
void or_backend_free(or_backend *b);
int32_t or_backend_n_threads(const or_backend *b);
int64_t or_backend_build_neighbor_list(or_backend *b, double *px, double *py, double *pz);
int64_t or_backend_pairs(const or_backend *b, const uint32_t **pair_i, const uint32_t **pair_j);
/* Installs a pair list (and its build positions) without running the O(N^2)
 * build; callers pass the reference's own pair set (e.g. from the cell path). */
int64_t or_backend_set_pairs(or_backend *b, int64_t n_pairs, const uint32_t *pair_i, const uint32_t *pair_j,
                             const double *px, const double *py, const double *pz);
/* cpu_backend.rs:92-182: fills f* (reduced buffer) and returns the energy. */
double or_backend_compute_forces(or_backend *b, const double *px, const double *py, const double *pz,
                                 double *fx, double *fy, double *fz);
int32_t or_backend_needs_rebuild(const or_backend *b, const double *px, const double *py, const double *pz);
int64_t or_backend_geodesic_drift(or_backend *b, double *px, double *py, double *pz,
                                  double *vx, double *vy, double *vz, double dt, uint64_t step,
                                  or_convergence_error *err);

/* geodesic/src/lib.rs:187-333, the BAB + RATTLE loop with the CPU backend.
 * Runs n_steps from (p*, v*) in place; every frame_interval steps (and at
 * step 0) it stores float32 positions (3 x n per frame, the DCD frame of
 * lib.rs:347-361), the potential and kinetic energy.  Returns the frame count,
 * or -1 (convergence error, *err set), -2 (non-finite force), -3
 * (non-finite position); *fail_step gets the failing step. */
int64_t or_run(const or_atoms *a, const or_topology *t, const or_params *p,
               double *px, double *py, double *pz, double *vx, double *vy, double *vz,
               double dt, uint64_t n_steps, uint32_t frame_interval, int64_t max_frames,
               float *frames, double *pot, double *kin, uint64_t *fail_step, or_convergence_error *err);

/* Host cores available to the CPU baseline. */
int32_t or_host_threads(void);

#ifdef __cplusplus
}
#endif
#endif
