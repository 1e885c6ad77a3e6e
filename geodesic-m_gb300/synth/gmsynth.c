/*
 * gmsynth.c — seeded synthetic MD systems for the CUDA backend's tests and
 * benchmarks (the jittered-lattice serpentine-chain systems the throughput
 * figures are quoted on).
 *
 * Geometry: atoms on a cubic lattice (spacing 2.15 A, 0.1 atoms/A^3),
 * uniform jitter +-0.3 A per coordinate.  The chain follows a serpentine
 * (boustrophedon) path through the lattice, so path neighbours are lattice
 * neighbours.  Bonds: path pairs (k = 300 kcal/mol/A^2, r0 = ideal lattice
 * distance).  Angles: path triples (k = 50 kcal/mol/rad^2, theta0 = ideal
 * lattice angle).  Dihedrals: path quads (k = 1 kcal/mol, n = 3, delta = 0;
 * k = 0 where either lattice angle of the quad is straight).
 * Exclusions: 1-2, 1-3 and 1-4 path pairs (AMBER lists 1-4 pairs as
 * excluded; a scaled 1-4 term adds them back when enabled).  Nonbonded:
 * 8 types, sigma U[2.0, 3.8] A, epsilon U[0.02, 0.2] kcal/mol, mass
 * U[12, 16] amu; charges U[-0.5, 0.5] e shifted to net zero.  Velocities:
 * Maxwell-Boltzmann at the requested temperature, zero net momentum.
 *
 * Optional hydrogens (h_fraction > 0): that fraction of lattice sites become
 * H atoms (mass 1.008; AMBER aliphatic-H Lennard-Jones, sigma 2.65 A,
 * epsilon 0.0157 kcal/mol; charges U[-0.1, 0.1] e, so that oppositely
 * charged H pairs cannot collapse onto each other; name "H"), each bonded
 * to a random lattice-adjacent heavy atom at 1.09 A (k = 340); the heavy
 * atoms keep the serpentine chain.  H atoms get H-X-Y angles to the
 * parent's chain neighbours and H-X-H angles to the parent's other H atoms
 * (k = 35) and the matching 1-2/1-3 exclusions.  The minimiser keeps the H bonds rigid
 * at 1.09 A and the velocities get no H-parent component along the bond,
 * so the MD run (H bonds constrained) starts on the constraint manifold.
 *
 * Pre-relaxation: FIRE minimisation in FP64 of bonds, angles, the scaled 1-4
 * pairs (LJ x 1/2, Coulomb x 1/1.2) and LJ + Coulomb with the quintic switch
 * over [8, 10] A -- the MD potential without dihedrals (at most relax_iters iterations,
 * stopping when the largest force is below 1 kcal/mol/A).  The lattice's
 * sigma range is wide for its 2.15 A spacing, so without it the compression
 * energy heats the system to thousands of kelvin and the droplet flies apart
 * in vacuum.  Deterministic for any thread count (gather per atom, fixed
 * order).  Everything derives from the 64-bit seed (splitmix64).
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SPACING 2.15
#define NTYPES 8

typedef struct {
    uint64_t s;
} rng_t;

static uint64_t splitmix(rng_t *r) {
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double uni(rng_t *r) { return (double)(splitmix(r) >> 11) * (1.0 / 9007199254740992.0); }
static double normal(rng_t *r) {
    double u1 = uni(r), u2 = uni(r);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

/* Output sizes for a request, so the caller can allocate. */
typedef struct {
    int64_t n_atoms, n_bonds, n_angles, n_diheds, n_excl, n_types;
} gs_sizes;

typedef struct {
    int64_t n_atoms;
    uint64_t seed;
    double h_fraction;
    double temperature;
    int32_t relax_iters;
    int32_t n_threads;
} gs_request;

typedef struct {
    /* per atom */
    double *pos;     /* 3 x N (x row, y row, z row) */
    double *vel;     /* 3 x N */
    double *sigma, *epsilon, *mass, *charge;
    uint8_t *element;  /* 0 = H, 1 = C */
    int32_t *type;
    /* topology */
    uint32_t *bond_i, *bond_j; double *bond_k, *bond_r0;
    uint32_t *angle_i, *angle_j, *angle_k; double *angle_kth, *angle_th0;
    uint32_t *dihed_i, *dihed_j, *dihed_k, *dihed_l; double *dihed_kphi; uint32_t *dihed_n; double *dihed_delta;
    uint32_t *excl_i, *excl_j;
    /* relaxation report */
    double max_force_before, max_force_after;
} gs_out;

static int side_for(int64_t n) {
    int s = (int)ceil(cbrt((double)n));
    while ((int64_t)s * s * s < n) s++;
    while (s > 1 && (int64_t)(s - 1) * (s - 1) * (s - 1) >= n) s--;
    return s;
}

/* serpentine lattice coordinate of path index p: rows run along x with the
 * direction flipping on every row (global row counter g), and the row order
 * flips on every plane, so the last site of a plane sits directly below the
 * first site of the next one. */
static void path_site(int64_t p, int side, int c[3]) {
    int64_t plane = (int64_t)side * side;
    int z = (int)(p / plane);
    int64_t k = p % plane;
    int yi = (int)(k / side);
    int xi = (int)(k % side);
    int y = (z & 1) ? side - 1 - yi : yi;
    int64_t g = (int64_t)z * side + yi;
    int x = (g & 1) ? side - 1 - xi : xi;
    c[0] = x; c[1] = y; c[2] = z;
}

static int64_t site_index(const int c[3], int side) { return ((int64_t)c[2] * side + c[1]) * side + c[0]; }

/* Builds the H designation and heavy-chain order; returns counts. */
typedef struct {
    int side;
    int64_t n;
    int64_t *site_of_atom;    /* lattice site of each atom (atoms in path order) */
    uint8_t *is_h;
    int64_t *h_parent;        /* heavy atom each H bonds to (atom index) */
    int64_t *heavy;           /* heavy atoms in chain order */
    int64_t n_heavy;
} layout_t;

static void make_layout(const gs_request *q, layout_t *L) {
    int64_t n = q->n_atoms;
    int side = side_for(n);
    L->side = side;
    L->n = n;
    L->site_of_atom = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    L->is_h = (uint8_t *)calloc((size_t)n, 1);
    L->h_parent = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    L->heavy = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int64_t nsite = (int64_t)side * side * side;
    int64_t *atom_at = (int64_t *)malloc(sizeof(int64_t) * (size_t)nsite);
    for (int64_t s = 0; s < nsite; s++) atom_at[s] = -1;
    int c[3];
    for (int64_t p = 0; p < n; p++) {
        path_site(p, side, c);
        L->site_of_atom[p] = site_index(c, side);
        atom_at[L->site_of_atom[p]] = p;
        L->h_parent[p] = -1;
    }
    if (q->h_fraction > 0.0) {
        /* H sites: random order over path positions; a site becomes H when
         * neither path neighbour is H (so the heavy chain keeps gaps of at
         * most one site) and it is not a chain end.  Random sequential
         * choice of this kind jams near 43% coverage, above 40%. */
        rng_t r = {q->seed ^ 0x48594452ull};
        int64_t want = (int64_t)llround(q->h_fraction * (double)n);
        int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
        for (int64_t i = 0; i < n; i++) order[i] = i;
        for (int64_t i = n - 1; i > 0; i--) {
            int64_t j = (int64_t)(uni(&r) * (double)(i + 1));
            if (j > i) j = i;
            int64_t t = order[i]; order[i] = order[j]; order[j] = t;
        }
        int64_t made = 0;
        for (int64_t k = 0; k < n && made < want; k++) {
            int64_t a = order[k];
            if (a == 0 || a == n - 1 || L->is_h[a - 1] || L->is_h[a + 1]) continue;
            L->is_h[a] = 1;
            made++;
        }
        /* parents: a random heavy lattice neighbour (path neighbours are
         * heavy lattice neighbours, so one always exists) */
        static const int dirs[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        for (int64_t a = 0; a < n; a++) {
            if (!L->is_h[a]) continue;
            int64_t s = L->site_of_atom[a];
            int cc[3] = {(int)(s % side), (int)((s / side) % side), (int)(s / ((int64_t)side * side))};
            int64_t cand[6];
            int nc = 0;
            for (int t = 0; t < 6; t++) {
                const int *d = dirs[t];
                int nb[3] = {cc[0] + d[0], cc[1] + d[1], cc[2] + d[2]};
                if (nb[0] < 0 || nb[1] < 0 || nb[2] < 0 || nb[0] >= side || nb[1] >= side || nb[2] >= side) continue;
                int64_t b = atom_at[site_index(nb, side)];
                if (b >= 0 && !L->is_h[b]) cand[nc++] = b;
            }
            int pick = (int)(uni(&r) * nc);
            if (pick >= nc) pick = nc - 1;
            L->h_parent[a] = cand[pick];
        }
        free(order);
    }
    L->n_heavy = 0;
    for (int64_t p = 0; p < n; p++) if (!L->is_h[p]) L->heavy[L->n_heavy++] = p;
    free(atom_at);
}

static void free_layout(layout_t *L) {
    free(L->site_of_atom); free(L->is_h); free(L->h_parent); free(L->heavy);
}

int gs_sizes_for(const gs_request *q, gs_sizes *out) {
    layout_t L;
    make_layout(q, &L);
    int64_t nh = L.n_heavy, n = L.n, nH = n - nh;
    out->n_atoms = n;
    out->n_bonds = (nh > 0 ? nh - 1 : 0) + nH;
    /* chain angles + one H-X-Y angle per chain neighbour Y of the parent */
    int64_t h_angles = 0;
    int64_t *pos_in_chain = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t k = 0; k < nh; k++) pos_in_chain[L.heavy[k]] = k;
    int64_t *nh_of = (int64_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int64_t));
    for (int64_t a = 0; a < n; a++) {
        if (!L.is_h[a]) continue;
        int64_t k = pos_in_chain[L.h_parent[a]];
        h_angles += (k > 0) + (k + 1 < nh);
        /* and one H-X-H angle per pair of H atoms sharing the parent */
        h_angles += nh_of[L.h_parent[a]]++;
    }
    free(nh_of);
    out->n_angles = (nh > 1 ? nh - 2 : 0) + h_angles;
    out->n_diheds = nh > 2 ? nh - 3 : 0;
    /* exclusions: chain 1-2, 1-3, 1-4; H: parent (1-2) + H-Y and H-H (1-3) */
    out->n_excl = (nh > 0 ? nh - 1 : 0) + (nh > 1 ? nh - 2 : 0) + (nh > 2 ? nh - 3 : 0) + nH + h_angles;
    out->n_types = NTYPES + (nH > 0);
    free(pos_in_chain);
    free_layout(&L);
    return 0;
}

static double lattice_angle(const double a[3], const double b[3], const double c[3]) {
    double u[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]}, v[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
    double d = (u[0] * v[0] + u[1] * v[1] + u[2] * v[2]) /
               (sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) * sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
    if (d > 1) d = 1;
    if (d < -1) d = -1;
    return acos(d);
}

/* ----------------------------------------------------------- relaxation */

/* FIRE minimisation (Bitzek et al., PRL 97, 170201 (2006)) of the MD
 * potential without dihedrals: bonds, angles, scaled 1-4 pairs, and LJ plus
 * Coulomb switched over [RELAX_SWITCH, RELAX_CUT].  Nonbonded pairs come from a Verlet list (cutoff +
 * RELAX_SKIN, rebuilt when an atom moved RELAX_SKIN/2); each atom gathers its
 * own neighbours in a fixed order, so the result does not depend on the
 * thread count. */
#define RELAX_SKIN 1.5
#define COUL_K 332.0522173

typedef struct {
    int64_t n;
    double rc, rs;  /* cutoff and switch onset of this stage */
    const double *pos, *sigma, *epsilon, *charge;
    const int64_t *nb_start;
    const uint32_t *nb;
    double *force;
    double *energy;   /* per thread */
    int64_t a0, a1;
    int t;
} nb_job;

static void *nb_worker(void *arg) {
    nb_job *J = (nb_job *)arg;
    int64_t n = J->n;
    const double *x = J->pos, *y = J->pos + n, *z = J->pos + 2 * n;
    const double rc2 = J->rc * J->rc, RELAX_CUT = J->rc, RELAX_SWITCH = J->rs;
    double e = 0.0;
    for (int64_t i = J->a0; i < J->a1; i++) {
        double f[3] = {0, 0, 0};
        for (int64_t m = J->nb_start[i]; m < J->nb_start[i + 1]; m++) {
            uint32_t j = J->nb[m];
            double dx = x[j] - x[i], dy = y[j] - y[i], dz = z[j] - z[i];
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > rc2 || r2 == 0.0) continue;
            /* the MD potential: LJ + Coulomb, quintic switch over [8, 10] A */
            double sg = 0.5 * (J->sigma[i] + J->sigma[j]);
            double ep = sqrt(J->epsilon[i] * J->epsilon[j]);
            double r = sqrt(r2);
            double s2 = sg * sg / r2, s6 = s2 * s2 * s2;
            double qq = COUL_K * J->charge[i] * J->charge[j];
            double v = 4.0 * ep * (s6 * s6 - s6) + qq / r;
            double fr = 24.0 * ep * (2.0 * s6 * s6 - s6) / r + qq / r2;   /* F_r */
            if (r > RELAX_SWITCH) {
                double u = (r - RELAX_SWITCH) / (RELAX_CUT - RELAX_SWITCH), u2 = u * u;
                double sw = 1.0 - 10.0 * u2 * u + 15.0 * u2 * u2 - 6.0 * u2 * u2 * u;
                double dsw = -30.0 * u2 * (1.0 - u) * (1.0 - u) / (RELAX_CUT - RELAX_SWITCH);
                fr = fr * sw - v * dsw;
                v *= sw;
            }
            fr /= r;
            e += 0.5 * v;
            f[0] -= fr * dx; f[1] -= fr * dy; f[2] -= fr * dz;
        }
        J->force[i] += f[0]; J->force[n + i] += f[1]; J->force[2 * n + i] += f[2];
    }
    J->energy[J->t] = e;
    return NULL;
}

static int excluded(const uint64_t *keys, int64_t nk, uint32_t i, uint32_t j) {
    if (i > j) { uint32_t t = i; i = j; j = t; }
    uint64_t k = ((uint64_t)i << 32) | j;
    int64_t lo = 0, hi = nk - 1;
    while (lo <= hi) {
        int64_t m = (lo + hi) >> 1;
        if (keys[m] == k) return 1;
        if (keys[m] < k) lo = m + 1; else hi = m - 1;
    }
    return 0;
}

static int cmp64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* full Verlet list within RELAX_CUT + RELAX_SKIN, exclusions removed */
static void build_verlet(int64_t n, const double *pos, const uint64_t *keys, int64_t nk, int64_t **start_out,
                         uint32_t **nb_out, int64_t *cap, double rc) {
    const double rl = rc + RELAX_SKIN, rl2 = rl * rl;
    double lo[3], hi[3], w[3];
    int nc[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = INFINITY; hi[d] = -INFINITY;
        for (int64_t i = 0; i < n; i++) { double v = pos[d * n + i]; if (v < lo[d]) lo[d] = v; if (v > hi[d]) hi[d] = v; }
        nc[d] = (int)floor((hi[d] - lo[d]) / (rl * 1.001));
        if (nc[d] < 1) nc[d] = 1;
        if (nc[d] > 256) nc[d] = 256;
        w[d] = (hi[d] - lo[d]) / nc[d];
        if (w[d] <= 0) w[d] = 1.0;
    }
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    int64_t *cs = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
    int64_t *cof = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int64_t *cat = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        int c3[3];
        for (int d = 0; d < 3; d++) {
            int c = (int)floor((pos[d * n + i] - lo[d]) / w[d]);
            c3[d] = c < 0 ? 0 : (c >= nc[d] ? nc[d] - 1 : c);
        }
        cof[i] = ((int64_t)c3[2] * nc[1] + c3[1]) * nc[0] + c3[0];
        cs[cof[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; c++) cs[c + 1] += cs[c];
    int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)ncell);
    memcpy(cur, cs, sizeof(int64_t) * (size_t)ncell);
    for (int64_t i = 0; i < n; i++) cat[cur[cof[i]]++] = i;  /* ascending i within a cell */
    free(cur);
    int64_t *start = *start_out;
    uint32_t *nb = *nb_out;
    int64_t used = 0;
    for (int64_t i = 0; i < n; i++) {
        start[i] = used;
        int64_t c = cof[i];
        int ci[3] = {(int)(c % nc[0]), (int)((c / nc[0]) % nc[1]), (int)(c / ((int64_t)nc[0] * nc[1]))};
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int cx = ci[0] + dx, cy = ci[1] + dy, cz = ci[2] + dz;
                    if (cx < 0 || cy < 0 || cz < 0 || cx >= nc[0] || cy >= nc[1] || cz >= nc[2]) continue;
                    int64_t cell = ((int64_t)cz * nc[1] + cy) * nc[0] + cx;
                    for (int64_t m = cs[cell]; m < cs[cell + 1]; m++) {
                        int64_t j = cat[m];
                        if (j == i) continue;
                        double ddx = pos[j] - pos[i], ddy = pos[n + j] - pos[n + i], ddz = pos[2 * n + j] - pos[2 * n + i];
                        if (ddx * ddx + ddy * ddy + ddz * ddz > rl2) continue;
                        if (nk && excluded(keys, nk, (uint32_t)i, (uint32_t)j)) continue;
                        if (used == *cap) {
                            *cap = *cap * 2 + 1024;
                            nb = (uint32_t *)realloc(nb, sizeof(uint32_t) * (size_t)*cap);
                        }
                        nb[used++] = (uint32_t)j;
                    }
                }
    }
    start[n] = used;
    *nb_out = nb;
    free(cs); free(cof); free(cat);
}

static double bonded_relax_forces(int64_t n, const double *p, const gs_sizes *S, const gs_out *o, double *F) {
    const double *x = p, *y = p + n, *z = p + 2 * n;
    double e = 0.0;
    /* 1-4 path pairs are excluded from the nonbonded list but interact
     * through the scaled 1-4 term (LJ x 1/2); at serpentine U-turns they are
     * lattice neighbours, so the relaxation must keep them apart too */
    for (int64_t d = 0; d < S->n_diheds; d++) {
        uint32_t i = o->dihed_i[d], j = o->dihed_l[d];
        double dd[3] = {x[j] - x[i], y[j] - y[i], z[j] - z[i]};
        double r2 = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
        if (r2 == 0.0) continue;
        double sg = 0.5 * (o->sigma[i] + o->sigma[j]), ep = sqrt(o->epsilon[i] * o->epsilon[j]);
        double s2 = sg * sg / r2, s6 = s2 * s2 * s2;
        double qq = COUL_K * o->charge[i] * o->charge[j] / 1.2;
        double r = sqrt(r2);
        double fr = 0.5 * 24.0 * ep * (2.0 * s6 * s6 - s6) / r2 + qq / (r2 * r);
        e += 0.5 * 4.0 * ep * (s6 * s6 - s6) + qq / r;
        for (int c = 0; c < 3; c++) { F[c * n + i] -= fr * dd[c]; F[c * n + j] += fr * dd[c]; }
    }
    for (int64_t b = 0; b < S->n_bonds; b++) {
        uint32_t i = o->bond_i[b], j = o->bond_j[b];
        double d[3] = {x[j] - x[i], y[j] - y[i], z[j] - z[i]};
        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (r == 0) continue;
        double g = 2.0 * o->bond_k[b] * (r - o->bond_r0[b]) / r;
        e += o->bond_k[b] * (r - o->bond_r0[b]) * (r - o->bond_r0[b]);
        for (int c = 0; c < 3; c++) { F[c * n + i] += g * d[c]; F[c * n + j] -= g * d[c]; }
    }
    for (int64_t a = 0; a < S->n_angles; a++) {
        uint32_t i = o->angle_i[a], j = o->angle_j[a], k = o->angle_k[a];
        if (o->angle_kth[a] == 0.0) continue;
        double b1[3] = {x[i] - x[j], y[i] - y[j], z[i] - z[j]}, b2[3] = {x[k] - x[j], y[k] - y[j], z[k] - z[j]};
        double r1 = sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
        double r2 = sqrt(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
        if (r1 == 0 || r2 == 0) continue;
        double ct = (b1[0] * b2[0] + b1[1] * b2[1] + b1[2] * b2[2]) / (r1 * r2);
        if (ct > 1) ct = 1;
        if (ct < -1) ct = -1;
        double st = sqrt(1 - ct * ct);
        if (st < 1e-3) st = 1e-3;
        double dth = acos(ct) - o->angle_th0[a];
        e += o->angle_kth[a] * dth * dth;
        double g = 2.0 * o->angle_kth[a] * dth / st;
        for (int c = 0; c < 3; c++) {
            double fi = g * (b2[c] / (r1 * r2) - ct * b1[c] / (r1 * r1));
            double fk = g * (b1[c] / (r1 * r2) - ct * b2[c] / (r2 * r2));
            F[c * n + i] += fi; F[c * n + k] += fk; F[c * n + j] -= fi + fk;
        }
    }
    return e;
}

/* Rigid H bonds inside the minimiser: the force on an H along its bond is
 * carried by the bond to the parent, and the H is put back at 1.09 A after
 * every move, so the minimum is taken on the constraint manifold (the MD run
 * then starts without a perpendicular load the constraints cannot take). */
static void rigid_h_forces(int64_t n, const double *pos, const int64_t *hp, double *F, double *V) {
    for (int64_t a = 0; a < n; a++) {
        const int64_t b = hp[a];
        if (b < 0) continue;
        double u[3], len = 0.0;
        for (int k = 0; k < 3; k++) { u[k] = pos[k * n + a] - pos[k * n + b]; len += u[k] * u[k]; }
        len = sqrt(len);
        if (!(len > 0.0)) continue;
        double fu = 0.0, vr = 0.0;
        for (int k = 0; k < 3; k++) {
            u[k] /= len;
            fu += F[k * n + a] * u[k];
            vr += (V[k * n + a] - V[k * n + b]) * u[k];
        }
        for (int k = 0; k < 3; k++) {
            F[k * n + a] -= fu * u[k];
            F[k * n + b] += fu * u[k];
            V[k * n + a] -= vr * u[k];
        }
    }
}

static void rigid_h_snap(int64_t n, double *pos, const int64_t *hp) {
    for (int64_t a = 0; a < n; a++) {
        const int64_t b = hp[a];
        if (b < 0) continue;
        double d[3], len = 0.0;
        for (int k = 0; k < 3; k++) { d[k] = pos[k * n + a] - pos[k * n + b]; len += d[k] * d[k]; }
        len = sqrt(len);
        if (len > 0.0)
            for (int k = 0; k < 3; k++) pos[k * n + a] = pos[k * n + b] + 1.09 * d[k] / len;
    }
}

static double relax_stage(int64_t n, double *pos, const gs_sizes *S, const gs_out *o, int iters, int n_threads,
                          double rc, double rs, double ftol, double *max_before, const int64_t *hp) {
    int64_t nk = S->n_excl;
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(nk > 0 ? nk : 1));
    for (int64_t e = 0; e < nk; e++) {
        uint32_t i = o->excl_i[e], j = o->excl_j[e];
        if (i > j) { uint32_t t = i; i = j; j = t; }
        keys[e] = ((uint64_t)i << 32) | j;
    }
    qsort(keys, (size_t)nk, sizeof(uint64_t), cmp64);
    if (n_threads < 1) n_threads = 1;
    double *F = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *V = (double *)calloc(3 * (size_t)n, sizeof(double));
    double *ref = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    int64_t *start = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    int64_t cap = n * 640 + 1024;
    uint32_t *nb = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)cap);
    double *eth = (double *)calloc((size_t)n_threads, sizeof(double));
    nb_job *jobs = (nb_job *)malloc(sizeof(nb_job) * (size_t)n_threads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
    build_verlet(n, pos, keys, nk, &start, &nb, &cap, rc);
    memcpy(ref, pos, sizeof(double) * 3 * (size_t)n);
    const double dt_max = 0.1, f_inc = 1.1, f_dec = 0.5, a_start = 0.1, f_a = 0.99, max_step = 0.1;
    double dt = 0.01, alpha = a_start, maxf = 0.0;
    int n_pos = 0;
    for (int it = 0; it <= iters; it++) {
        /* rebuild the list once an atom moved half the skin */
        double dmax = 0.0;
        for (int64_t i = 0; i < n; i++) {
            double dx = pos[i] - ref[i], dy = pos[n + i] - ref[n + i], dz = pos[2 * n + i] - ref[2 * n + i];
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > dmax) dmax = d2;
        }
        if (dmax > 0.25 * RELAX_SKIN * RELAX_SKIN) {
            build_verlet(n, pos, keys, nk, &start, &nb, &cap, rc);
            memcpy(ref, pos, sizeof(double) * 3 * (size_t)n);
        }
        memset(F, 0, sizeof(double) * 3 * (size_t)n);
        bonded_relax_forces(n, pos, S, o, F);
        int64_t chunk = (n + n_threads - 1) / n_threads;
        for (int t = 0; t < n_threads; t++) {
            nb_job J = {n, rc, rs, pos, o->sigma, o->epsilon, o->charge, start, nb, F, eth, t * chunk, (t + 1) * chunk, t};
            if (J.a0 > n) J.a0 = n;
            if (J.a1 > n) J.a1 = n;
            jobs[t] = J;
            if (t > 0) pthread_create(&th[t], NULL, nb_worker, &jobs[t]);
        }
        nb_worker(&jobs[0]);
        for (int t = 1; t < n_threads; t++) pthread_join(th[t], NULL);
        if (hp) rigid_h_forces(n, pos, hp, F, V);
        maxf = 0.0;
        double P = 0.0, fn = 0.0, vn = 0.0;
        for (int64_t i = 0; i < 3 * n; i++) { P += F[i] * V[i]; fn += F[i] * F[i]; vn += V[i] * V[i]; }
        for (int64_t i = 0; i < n; i++) {
            double f2 = F[i] * F[i] + F[n + i] * F[n + i] + F[2 * n + i] * F[2 * n + i];
            if (f2 > maxf) maxf = f2;
        }
        maxf = sqrt(maxf);
        if (it == 0 && max_before) *max_before = maxf;
        if (it == iters || maxf < ftol) break;
        /* FIRE velocity mixing and time-step control */
        if (P > 0.0) {
            double s = fn > 0 ? alpha * sqrt(vn / fn) : 0.0;
            for (int64_t i = 0; i < 3 * n; i++) V[i] = (1.0 - alpha) * V[i] + s * F[i];
            if (++n_pos > 5) { dt = dt * f_inc < dt_max ? dt * f_inc : dt_max; alpha *= f_a; }
        } else {
            memset(V, 0, sizeof(double) * 3 * (size_t)n);
            dt *= f_dec;
            alpha = a_start;
            n_pos = 0;
        }
        for (int64_t i = 0; i < n; i++) {
            double d[3];
            double d2 = 0.0;
            for (int c = 0; c < 3; c++) { V[c * n + i] += dt * F[c * n + i]; d[c] = dt * V[c * n + i]; d2 += d[c] * d[c]; }
            double sc = d2 > max_step * max_step ? max_step / sqrt(d2) : 1.0;
            for (int c = 0; c < 3; c++) pos[c * n + i] += sc * d[c];
        }
        if (hp) rigid_h_snap(n, pos, hp);
    }
    free(F); free(V); free(ref); free(start); free(nb); free(eth); free(jobs); free(th); free(keys);
    return maxf;
}

/* Two stages: most iterations on the cheap 6 A switched potential, then a
 * fifth of them on the full potential (switch 8 -> 10 A). */
static double relax(int64_t n, double *pos, const gs_sizes *S, const gs_out *o, int iters, int n_threads,
                    double *max_before, const int64_t *hp) {
    if (hp) rigid_h_snap(n, pos, hp);
    if (iters <= 0) return relax_stage(n, pos, S, o, 0, n_threads, 10.0, 8.0, 1.0, max_before, hp);
    int polish = iters / 5 > 0 ? iters / 5 : 1;
    relax_stage(n, pos, S, o, iters - polish, n_threads, 6.0, 4.0, 0.5, max_before, hp);
    return relax_stage(n, pos, S, o, polish, n_threads, 10.0, 8.0, 1.0, NULL, hp);
}

/* ------------------------------------------------------------ generate */

int gs_generate(const gs_request *q, const gs_sizes *S, gs_out *o) {
    layout_t L;
    make_layout(q, &L);
    int64_t n = L.n, nh = L.n_heavy;
    int side = L.side;
    rng_t r = {q->seed};
    /* types */
    double tsig[NTYPES + 1], teps[NTYPES + 1], tmass[NTYPES + 1];
    for (int t = 0; t < NTYPES; t++) {
        tsig[t] = 2.0 + 1.8 * uni(&r);
        teps[t] = 0.02 + 0.18 * uni(&r);
        tmass[t] = 12.0 + 4.0 * uni(&r);
    }
    tsig[NTYPES] = 2.65; teps[NTYPES] = 0.0157; tmass[NTYPES] = 1.008;
    double qsum = 0.0;
    int c[3];
    double *x = o->pos, *y = o->pos + n, *z = o->pos + 2 * n;
    for (int64_t p = 0; p < n; p++) {
        int s = (int)(uni(&r) * NTYPES);
        if (s >= NTYPES) s = NTYPES - 1;
        if (L.is_h[p]) s = NTYPES;
        o->type[p] = s;
        o->sigma[p] = tsig[s];
        o->epsilon[p] = teps[s];
        o->mass[p] = tmass[s];
        o->element[p] = L.is_h[p] ? 0 : 1;
        o->charge[p] = L.is_h[p] ? 0.2 * (uni(&r) - 0.5) : -0.5 + uni(&r);
        qsum += o->charge[p];
        path_site(p, side, c);
        x[p] = c[0] * SPACING + (uni(&r) * 0.6 - 0.3);
        y[p] = c[1] * SPACING + (uni(&r) * 0.6 - 0.3);
        z[p] = c[2] * SPACING + (uni(&r) * 0.6 - 0.3);
    }
    double qmean = n > 0 ? qsum / (double)n : 0.0;
    for (int64_t p = 0; p < n; p++) o->charge[p] -= qmean;
    /* ideal lattice positions, for r0 / theta0 */
    double *ideal = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    for (int64_t p = 0; p < n; p++) {
        path_site(p, side, c);
        for (int d = 0; d < 3; d++) ideal[3 * p + d] = c[d] * SPACING;
    }
    /* H atoms sit 1.09 A from their parent, along the lattice direction */
    for (int64_t a = 0; a < n; a++) {
        if (!L.is_h[a]) continue;
        int64_t b = L.h_parent[a];
        double d[3], len = 0;
        for (int k = 0; k < 3; k++) { d[k] = ideal[3 * a + k] - ideal[3 * b + k]; len += d[k] * d[k]; }
        len = sqrt(len);
        double pb[3] = {x[b], y[b], z[b]};
        x[a] = pb[0] + 1.09 * d[0] / len;
        y[a] = pb[1] + 1.09 * d[1] / len;
        z[a] = pb[2] + 1.09 * d[2] / len;
        for (int k = 0; k < 3; k++) ideal[3 * a + k] = ideal[3 * b + k] + 1.09 * d[k] / len;
    }
    int64_t nb = 0, na = 0, nd = 0, ne = 0;
    for (int64_t k = 0; k + 1 < nh; k++) {
        int64_t i = L.heavy[k], j = L.heavy[k + 1];
        double rr = 0;
        for (int d = 0; d < 3; d++) rr += (ideal[3 * j + d] - ideal[3 * i + d]) * (ideal[3 * j + d] - ideal[3 * i + d]);
        o->bond_i[nb] = (uint32_t)i; o->bond_j[nb] = (uint32_t)j; o->bond_k[nb] = 300.0; o->bond_r0[nb] = sqrt(rr); nb++;
    }
    int64_t *pos_in_chain = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t k = 0; k < nh; k++) pos_in_chain[L.heavy[k]] = k;
    for (int64_t a = 0; a < n; a++) {
        if (!L.is_h[a]) continue;
        o->bond_i[nb] = (uint32_t)L.h_parent[a]; o->bond_j[nb] = (uint32_t)a; o->bond_k[nb] = 340.0; o->bond_r0[nb] = 1.09; nb++;
    }
    for (int64_t k = 0; k + 2 < nh; k++) {
        int64_t i = L.heavy[k], j = L.heavy[k + 1], l = L.heavy[k + 2];
        o->angle_i[na] = (uint32_t)i; o->angle_j[na] = (uint32_t)j; o->angle_k[na] = (uint32_t)l;
        o->angle_kth[na] = 50.0; o->angle_th0[na] = lattice_angle(&ideal[3 * i], &ideal[3 * j], &ideal[3 * l]); na++;
    }
    for (int64_t a = 0; a < n; a++) {
        if (!L.is_h[a]) continue;
        int64_t b = L.h_parent[a], k = pos_in_chain[b];
        for (int side_ = 0; side_ < 2; side_++) {
            int64_t kk = side_ == 0 ? k - 1 : k + 1;
            if (kk < 0 || kk >= nh) continue;
            int64_t yv = L.heavy[kk];
            o->angle_i[na] = (uint32_t)a; o->angle_j[na] = (uint32_t)b; o->angle_k[na] = (uint32_t)yv;
            double th = lattice_angle(&ideal[3 * a], &ideal[3 * b], &ideal[3 * yv]);
            /* H on the X-Y line (ideal angle 0 or 180 deg) is a degenerate
             * angle term: keep it in the topology with zero force constant */
            int degenerate = th < 0.2 || th > M_PI - 0.2;
            o->angle_kth[na] = degenerate ? 0.0 : 35.0; o->angle_th0[na] = th; na++;
            o->excl_i[ne] = (uint32_t)(a < yv ? a : yv); o->excl_j[ne] = (uint32_t)(a < yv ? yv : a); ne++;
        }
        /* H-X-H with every earlier H of the same parent (as a force field's
         * H-C-H angles): keeps the H atoms of one parent apart and excludes
         * their 1-3 pair */
        for (int64_t e = 0; e < a; e++) {
            if (!L.is_h[e] || L.h_parent[e] != b) continue;
            o->angle_i[na] = (uint32_t)e; o->angle_j[na] = (uint32_t)b; o->angle_k[na] = (uint32_t)a;
            double th = lattice_angle(&ideal[3 * e], &ideal[3 * b], &ideal[3 * a]);
            int degenerate = th < 0.2 || th > M_PI - 0.2;
            o->angle_kth[na] = degenerate ? 0.0 : 35.0; o->angle_th0[na] = th; na++;
            o->excl_i[ne] = (uint32_t)e; o->excl_j[ne] = (uint32_t)a; ne++;
        }
    }
    for (int64_t k = 0; k + 3 < nh; k++) {
        const int64_t a0 = L.heavy[k], a1 = L.heavy[k + 1], a2 = L.heavy[k + 2], a3 = L.heavy[k + 3];
        o->dihed_i[nd] = (uint32_t)a0; o->dihed_j[nd] = (uint32_t)a1;
        o->dihed_k[nd] = (uint32_t)a2; o->dihed_l[nd] = (uint32_t)a3;
        /* a torsion about a straight (180 deg) lattice angle is undefined and
         * the cross-product forces diverge as the angle fluctuates through
         * 180 deg: such quads stay in the topology with zero barrier */
        const double t1 = lattice_angle(&ideal[3 * a0], &ideal[3 * a1], &ideal[3 * a2]);
        const double t2 = lattice_angle(&ideal[3 * a1], &ideal[3 * a2], &ideal[3 * a3]);
        const int straight = t1 > M_PI - 0.2 || t2 > M_PI - 0.2;
        o->dihed_kphi[nd] = straight ? 0.0 : 1.0; o->dihed_n[nd] = 3; o->dihed_delta[nd] = 0.0; nd++;
    }
    for (int sep = 1; sep <= 3; sep++)
        for (int64_t k = 0; k + sep < nh; k++) {
            int64_t i = L.heavy[k], j = L.heavy[k + sep];
            o->excl_i[ne] = (uint32_t)(i < j ? i : j); o->excl_j[ne] = (uint32_t)(i < j ? j : i); ne++;
        }
    for (int64_t a = 0; a < n; a++) {
        if (!L.is_h[a]) continue;
        int64_t b = L.h_parent[a];
        o->excl_i[ne] = (uint32_t)(a < b ? a : b); o->excl_j[ne] = (uint32_t)(a < b ? b : a); ne++;
    }
    free(pos_in_chain);
    free(ideal);
    if (nb != S->n_bonds || na != S->n_angles || nd != S->n_diheds || ne != S->n_excl) { free_layout(&L); return -1; }
    /* relaxation */
    /* with hydrogens the H bonds are rigid in the minimiser (they become
     * constraints in the MD run), so the start lies on the constraint
     * manifold without a load the constraints cannot take */
    int64_t *hp = NULL;
    if (q->h_fraction > 0.0) {
        hp = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
        for (int64_t a = 0; a < n; a++) hp[a] = L.is_h[a] ? L.h_parent[a] : -1;
    }
    o->max_force_after = relax(n, o->pos, S, o, q->relax_iters, q->n_threads, &o->max_force_before, hp);
    free(hp);
    /* Maxwell-Boltzmann velocities, zero net momentum */
    rng_t rv = {q->seed ^ 0x56454C4Full};
    const double kB = 0.0019872041; /* kcal/mol/K */
    double pm[3] = {0, 0, 0}, mt = 0;
    for (int64_t p = 0; p < n; p++) {
        double sd = sqrt(kB * q->temperature / o->mass[p] * (20.455 * 20.455));
        for (int d = 0; d < 3; d++) { o->vel[d * n + p] = q->temperature > 0 ? sd * normal(&rv) : 0.0; pm[d] += o->mass[p] * o->vel[d * n + p]; }
        mt += o->mass[p];
    }
    if (n > 0 && q->temperature > 0)
        for (int64_t p = 0; p < n; p++)
            for (int d = 0; d < 3; d++) o->vel[d * n + p] -= pm[d] / mt;
    /* and on its tangent space: no H-parent relative velocity along the bond
     * (only the H velocity changes, so H atoms sharing a parent stay
     * independent) */
    for (int64_t a = 0; a < n; a++) {
        if (!L.is_h[a]) continue;
        const int64_t b = L.h_parent[a];
        double u[3], len = 0.0, vr = 0.0;
        for (int k = 0; k < 3; k++) { u[k] = o->pos[k * n + a] - o->pos[k * n + b]; len += u[k] * u[k]; }
        len = sqrt(len);
        if (!(len > 0.0)) continue;
        for (int k = 0; k < 3; k++) { u[k] /= len; vr += (o->vel[k * n + a] - o->vel[k * n + b]) * u[k]; }
        for (int k = 0; k < 3; k++) o->vel[k * n + a] -= vr * u[k];
    }
    free_layout(&L);
    return 0;
}
