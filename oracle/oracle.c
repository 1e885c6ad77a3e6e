/*
 * oracle.c — CPU restatement of the GEODESIC-M reference engine (FP64).
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Each function follows the cited
 * reference code statement by statement; evaluation order is kept because
 * the reference promises bit-for-bit repeatability and the CUDA backend's
 * FP64 kernels are checked against these values.  Compiled with
 * -ffp-contract=off so a*b+c is never fused (Rust does not fuse either).
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ---------------------------------------------------------------- helpers */

/* neighbor.rs:74-76 — Rust f64::round is half-away-from-zero, i.e. C round(). */
double or_min_image(double d, double box_len) { return d - box_len * round(d / box_len); }

/* Beyond reference: with a box (periodic + bonded_min_image), the
 * displacement between the two atoms of a bond, an angle arm, a dihedral
 * bond vector, a 1-4 pair or a constraint goes to the nearest image with the
 * reference's min_image expression (neighbor.rs:74-76); the reference keeps
 * them raw (memory.md:140-144).  NULL box: the raw difference, unchanged. */
static double bdiff(double d, const double *mi_box, int c) { return mi_box ? or_min_image(d, mi_box[c]) : d; }

static const double *mi_box_of(const or_params *p) { return (p->periodic && p->bonded_min_image) ? p->box : NULL; }

/* neighbor.rs:86-88 */
double or_wrap_coord(double x, double box_len) { return x - box_len * floor(x / box_len); }

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* neighbor.rs:18-23: the exclusion set, normalised to (min, max). */
static uint64_t *exclusion_keys(const or_topology *t, int64_t *n_keys) {
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(t->n_excl > 0 ? t->n_excl : 1));
    for (int64_t e = 0; e < t->n_excl; e++) {
        uint32_t i = t->excl_i[e], j = t->excl_j[e];
        if (i > j) { uint32_t s = i; i = j; j = s; }
        keys[e] = ((uint64_t)i << 32) | j;
    }
    qsort(keys, (size_t)t->n_excl, sizeof(uint64_t), cmp_u64);
    *n_keys = t->n_excl;
    return keys;
}

static int is_excluded(const uint64_t *keys, int64_t n_keys, uint32_t i, uint32_t j) {
    uint64_t k = ((uint64_t)i << 32) | j;
    int64_t lo = 0, hi = n_keys - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) >> 1;
        if (keys[mid] == k) return 1;
        if (keys[mid] < k) lo = mid + 1; else hi = mid - 1;
    }
    return 0;
}

static void wrap_into_box(int64_t n, double *px, double *py, double *pz, const double box[3]) {
    /* neighbor.rs:78-84 */
    for (int64_t i = 0; i < n; i++) {
        px[i] = or_wrap_coord(px[i], box[0]);
        py[i] = or_wrap_coord(py[i], box[1]);
        pz[i] = or_wrap_coord(pz[i], box[2]);
    }
}

/* ------------------------------------------------------- neighbour list */

/* The pairs of neighbor.rs:25-43 over the (already wrapped) positions, all
 * i < j; at most cap are stored, the count is returned. */
static int64_t pairs_all(int64_t n, const double *px, const double *py, const double *pz, const or_params *p,
                         const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j) {
    int64_t nk;
    uint64_t *keys = exclusion_keys(t, &nk);
    /* neighbor.rs:25 */
    const double r_skin_sq = p->r_skin * p->r_skin;
    int64_t count = 0;
    /* neighbor.rs:29-43.  The reference probes the exclusion set before the
     * distance; testing the distance first yields the same set and order. */
    for (int64_t i = 0; i < n; i++) {
        for (int64_t j = i + 1; j < n; j++) {
            double dx = or_min_image(px[j] - px[i], p->box[0]);
            double dy = or_min_image(py[j] - py[i], p->box[1]);
            double dz = or_min_image(pz[j] - pz[i], p->box[2]);
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 <= r_skin_sq) {
                if (nk && is_excluded(keys, nk, (uint32_t)i, (uint32_t)j)) continue;
                if (count < cap) { pair_i[count] = (uint32_t)i; pair_j[count] = (uint32_t)j; }
                count++;
            }
        }
    }
    free(keys);
    return count;
}

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

/* The same pairs found through a cell grid (same set, same order). */
static int64_t pairs_cells(int64_t n, const double *px, const double *py, const double *pz, const or_params *p,
                           const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j) {
    int64_t nk;
    uint64_t *keys = exclusion_keys(t, &nk);
    const double r_skin_sq = p->r_skin * p->r_skin;
    /* grid over the bounding box (non-periodic) or the box (periodic); the
     * cell edge exceeds r_skin by a margin so every listed pair is in a
     * neighbouring cell under the reference's own FP64 test. */
    double lo[3], hi[3];
    const double *P[3] = {px, py, pz};
    int nc[3];
    int full[3];
    for (int d = 0; d < 3; d++) {
        if (p->periodic) { lo[d] = 0.0; hi[d] = p->box[d]; }
        else {
            lo[d] = INFINITY; hi[d] = -INFINITY;
            for (int64_t i = 0; i < n; i++) { if (P[d][i] < lo[d]) lo[d] = P[d][i]; if (P[d][i] > hi[d]) hi[d] = P[d][i]; }
            if (n == 0) { lo[d] = 0; hi[d] = 1; }
        }
        double edge = p->r_skin * 1.0000001 + 1e-9;
        int c = (int)floor((hi[d] - lo[d]) / edge);
        if (c < 1) c = 1;
        if (c > 1024) c = 1024;
        nc[d] = c;
        /* a periodic dimension with fewer than 3 cells is scanned whole */
        full[d] = p->periodic ? (c < 3) : 0;
        if (!p->periodic && (hi[d] - lo[d]) >= 0.5 * p->box[d] - p->r_skin) {
            /* min-image may fold far pairs: fall back to the double loop */
            free(keys);
            return pairs_all(n, px, py, pz, p, t, cap, pair_i, pair_j);
        }
    }
    int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    int64_t *cstart = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
    int64_t *cellof = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int cc[3];
    for (int64_t i = 0; i < n; i++) {
        for (int d = 0; d < 3; d++) {
            double w = (hi[d] - lo[d]) / nc[d];
            int c = (int)floor((P[d][i] - lo[d]) / w);
            if (c < 0) c = 0;
            if (c >= nc[d]) c = nc[d] - 1;
            cc[d] = c;
        }
        cellof[i] = ((int64_t)cc[2] * nc[1] + cc[1]) * nc[0] + cc[0];
        cstart[cellof[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; c++) cstart[c + 1] += cstart[c];
    int64_t *cursor = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncell > 0 ? ncell : 1));
    memcpy(cursor, cstart, sizeof(int64_t) * (size_t)ncell);
    uint32_t *members = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) members[cursor[cellof[i]]++] = (uint32_t)i;
    uint32_t *buf = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    int64_t count = 0;
    for (int64_t i = 0; i < n; i++) {
        int64_t c = cellof[i];
        int ci[3] = {(int)(c % nc[0]), (int)((c / nc[0]) % nc[1]), (int)(c / ((int64_t)nc[0] * nc[1]))};
        int64_t nb = 0;
        int rlo[3], rhi[3];
        for (int d = 0; d < 3; d++) {
            if (full[d]) { rlo[d] = 0; rhi[d] = nc[d] - 1; }
            else if (p->periodic) { rlo[d] = ci[d] - 1; rhi[d] = ci[d] + 1; }
            else { rlo[d] = ci[d] > 0 ? ci[d] - 1 : 0; rhi[d] = ci[d] + 1 < nc[d] ? ci[d] + 1 : nc[d] - 1; }
        }
        for (int z = rlo[2]; z <= rhi[2]; z++)
            for (int y = rlo[1]; y <= rhi[1]; y++)
                for (int x = rlo[0]; x <= rhi[0]; x++) {
                    int wx = ((x % nc[0]) + nc[0]) % nc[0], wy = ((y % nc[1]) + nc[1]) % nc[1], wz = ((z % nc[2]) + nc[2]) % nc[2];
                    int64_t cell = ((int64_t)wz * nc[1] + wy) * nc[0] + wx;
                    for (int64_t m = cstart[cell]; m < cstart[cell + 1]; m++) {
                        uint32_t j = members[m];
                        if (j <= (uint32_t)i) continue;
                        double dx = or_min_image(px[j] - px[i], p->box[0]);
                        double dy = or_min_image(py[j] - py[i], p->box[1]);
                        double dz = or_min_image(pz[j] - pz[i], p->box[2]);
                        double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 <= r_skin_sq && !(nk && is_excluded(keys, nk, (uint32_t)i, j))) buf[nb++] = j;
                    }
                }
        /* wrapped stencils can visit a cell twice when nc == 3 is not full;
         * sort + dedupe keeps the reference's (i, then j) order and set. */
        qsort(buf, (size_t)nb, sizeof(uint32_t), cmp_u32);
        for (int64_t k = 0; k < nb; k++) {
            if (k > 0 && buf[k] == buf[k - 1]) continue;
            if (count < cap) { pair_i[count] = (uint32_t)i; pair_j[count] = buf[k]; }
            count++;
        }
    }
    free(buf); free(members); free(cursor); free(cellof); free(cstart); free(keys);
    return count;
}

/* neighbor::build (neighbor.rs:8-55): wraps a periodic system into the box
 * once (neighbor.rs:13-15), then lists the pairs.  A caller that only learns
 * the count from this call fetches the pairs with or_neighbor_pairs, which
 * does not wrap again (a coordinate that the wrap put exactly on L would turn
 * into 0 on a second one, which the reference never does). */
int64_t or_neighbor_build(int64_t n, double *px, double *py, double *pz, const or_params *p,
                          const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j) {
    if (p->periodic) wrap_into_box(n, px, py, pz, p->box);
    return pairs_all(n, px, py, pz, p, t, cap, pair_i, pair_j);
}

int64_t or_neighbor_build_cells(int64_t n, double *px, double *py, double *pz, const or_params *p,
                                const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j) {
    if (p->periodic) wrap_into_box(n, px, py, pz, p->box);
    return pairs_cells(n, px, py, pz, p, t, cap, pair_i, pair_j);
}

int64_t or_neighbor_pairs(int64_t n, const double *px, const double *py, const double *pz, const or_params *p,
                          const or_topology *t, int64_t cap, uint32_t *pair_i, uint32_t *pair_j, int32_t cells) {
    return cells ? pairs_cells(n, px, py, pz, p, t, cap, pair_i, pair_j)
                 : pairs_all(n, px, py, pz, p, t, cap, pair_i, pair_j);
}

int32_t or_needs_rebuild(int64_t n, const double *px, const double *py, const double *pz,
                         const double *rx, const double *ry, const double *rz,
                         double r_skin, double r_cutoff) {
    /* neighbor.rs:60-72 */
    double half_skin = (r_skin - r_cutoff) / 2.0;
    double threshold_sq = half_skin * half_skin;
    for (int64_t i = 0; i < n; i++) {
        double dx = px[i] - rx[i];
        double dy = py[i] - ry[i];
        double dz = pz[i] - rz[i];
        if (dx * dx + dy * dy + dz * dz > threshold_sq) return 1;
    }
    return 0;
}

/* ----------------------------------------------------------- nonbonded */

double or_pair_forces(const double *px, const double *py, const double *pz, const or_atoms *a,
                      const uint32_t *pair_i, const uint32_t *pair_j, int64_t n_pairs,
                      double r_cutoff, double r_switch, const double box[3],
                      double *fx, double *fy, double *fz) {
    /* force/nonbonded.rs:20-82 */
    double potential = 0.0;
    for (int64_t k = 0; k < n_pairs; k++) {
        uint32_t i = pair_i[k], j = pair_j[k];
        double dx = or_min_image(px[j] - px[i], box[0]);
        double dy = or_min_image(py[j] - py[i], box[1]);
        double dz = or_min_image(pz[j] - pz[i], box[2]);
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > r_cutoff * r_cutoff || r2 == 0.0) continue;
        double r = sqrt(r2);
        double sigma = 0.5 * (a->sigma[i] + a->sigma[j]);
        double epsilon = sqrt(a->epsilon[i] * a->epsilon[j]);
        if (epsilon == 0.0) continue;
        /* (sigma / r).powi(6): LLVM expands powi by binary exponentiation,
         * x^6 = (x*x) * ((x*x)*(x*x)). */
        double s = sigma / r;
        double s2 = s * s;
        double s4 = s2 * s2;
        double sr6 = s2 * s4;
        double sr12 = sr6 * sr6;
        double v_lj = 4.0 * epsilon * (sr12 - sr6);
        double f_lj = 24.0 * epsilon / r * (2.0 * sr12 - sr6);
        double v, f_radial;
        if (r <= r_switch) {
            v = v_lj; f_radial = f_lj;
        } else {
            double u = (r - r_switch) / (r_cutoff - r_switch);
            double u2 = u * u;
            double sw = 1.0 - 10.0 * u2 * u + 15.0 * u2 * u2 - 6.0 * u2 * u2 * u;
            double ds_dr = -30.0 * u2 * (1.0 - u) * (1.0 - u) / (r_cutoff - r_switch);
            v = v_lj * sw;
            f_radial = f_lj * sw - v_lj * ds_dr;
        }
        potential += v;
        double gx = f_radial * dx / r;
        double gy = f_radial * dy / r;
        double gz = f_radial * dz / r;
        fx[i] -= gx; fy[i] -= gy; fz[i] -= gz;
        fx[j] += gx; fy[j] += gy; fz[j] += gz;
    }
    return potential;
}

#define COULOMB_KCAL 332.0522173

double or_coulomb_forces(const double *px, const double *py, const double *pz, const or_atoms *a,
                         const uint32_t *pair_i, const uint32_t *pair_j, int64_t n_pairs,
                         double r_cutoff, double r_switch, const double box[3],
                         double *fx, double *fy, double *fz) {
    /* beyond reference: V = k q_i q_j / r * S(r), same switch as the LJ term */
    double potential = 0.0;
    for (int64_t k = 0; k < n_pairs; k++) {
        uint32_t i = pair_i[k], j = pair_j[k];
        double dx = or_min_image(px[j] - px[i], box[0]);
        double dy = or_min_image(py[j] - py[i], box[1]);
        double dz = or_min_image(pz[j] - pz[i], box[2]);
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 > r_cutoff * r_cutoff || r2 == 0.0) continue;
        double r = sqrt(r2);
        double qq = COULOMB_KCAL * a->charge[i] * a->charge[j];
        if (qq == 0.0) continue;
        double v_c = qq / r;
        double f_c = qq / r2; /* -dV/dr */
        double v, f_radial;
        if (r <= r_switch) {
            v = v_c; f_radial = f_c;
        } else {
            double u = (r - r_switch) / (r_cutoff - r_switch);
            double u2 = u * u;
            double sw = 1.0 - 10.0 * u2 * u + 15.0 * u2 * u2 - 6.0 * u2 * u2 * u;
            double ds_dr = -30.0 * u2 * (1.0 - u) * (1.0 - u) / (r_cutoff - r_switch);
            v = v_c * sw;
            f_radial = f_c * sw - v_c * ds_dr;
        }
        potential += v;
        double gx = f_radial * dx / r, gy = f_radial * dy / r, gz = f_radial * dz / r;
        fx[i] -= gx; fy[i] -= gy; fz[i] -= gz;
        fx[j] += gx; fy[j] += gy; fz[j] += gz;
    }
    return potential;
}

int64_t or_pairs14(const or_topology *t, int64_t n_atoms, int64_t cap, uint32_t *p14_i, uint32_t *p14_j) {
    (void)n_atoms;
    int64_t nd = t->n_diheds;
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(nd > 0 ? nd : 1));
    int64_t m = 0;
    /* 1-2 and 1-3 pairs, to drop 1-4 candidates that are also closer neighbours */
    int64_t n13 = t->n_bonds + t->n_angles;
    uint64_t *close = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n13 > 0 ? n13 : 1));
    for (int64_t b = 0; b < t->n_bonds; b++) {
        uint32_t i = t->bond_i[b], j = t->bond_j[b];
        if (i > j) { uint32_t s = i; i = j; j = s; }
        close[b] = ((uint64_t)i << 32) | j;
    }
    for (int64_t g = 0; g < t->n_angles; g++) {
        uint32_t i = t->angle_i[g], j = t->angle_k[g];
        if (i > j) { uint32_t s = i; i = j; j = s; }
        close[t->n_bonds + g] = ((uint64_t)i << 32) | j;
    }
    qsort(close, (size_t)n13, sizeof(uint64_t), cmp_u64);
    for (int64_t d = 0; d < nd; d++) {
        uint32_t i = t->dihed_i[d], j = t->dihed_l[d];
        if (i == j) continue;
        if (i > j) { uint32_t s = i; i = j; j = s; }
        if (n13 && is_excluded(close, n13, i, j)) continue;
        keys[m++] = ((uint64_t)i << 32) | j;
    }
    qsort(keys, (size_t)m, sizeof(uint64_t), cmp_u64);
    int64_t count = 0;
    for (int64_t k = 0; k < m; k++) {
        if (k > 0 && keys[k] == keys[k - 1]) continue;
        if (count < cap) { p14_i[count] = (uint32_t)(keys[k] >> 32); p14_j[count] = (uint32_t)keys[k]; }
        count++;
    }
    free(keys); free(close);
    return count;
}

double or_pair14_forces_box(const double *px, const double *py, const double *pz, const or_atoms *a,
                            const uint32_t *p14_i, const uint32_t *p14_j, int64_t n14,
                            double scale_lj, double scale_coul, int32_t coulomb, const double *mi_box,
                            double *fx, double *fy, double *fz) {
    double potential = 0.0;
    for (int64_t k = 0; k < n14; k++) {
        uint32_t i = p14_i[k], j = p14_j[k];
        double dx = bdiff(px[j] - px[i], mi_box, 0), dy = bdiff(py[j] - py[i], mi_box, 1);
        double dz = bdiff(pz[j] - pz[i], mi_box, 2);
        double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 == 0.0) continue;
        double r = sqrt(r2);
        double v = 0.0, f_radial = 0.0;
        double sigma = 0.5 * (a->sigma[i] + a->sigma[j]);
        double epsilon = sqrt(a->epsilon[i] * a->epsilon[j]);
        if (scale_lj != 0.0 && epsilon != 0.0) {
            double s = sigma / r, s2 = s * s, s4 = s2 * s2, sr6 = s2 * s4, sr12 = sr6 * sr6;
            v += scale_lj * (4.0 * epsilon * (sr12 - sr6));
            f_radial += scale_lj * (24.0 * epsilon / r * (2.0 * sr12 - sr6));
        }
        if (coulomb && scale_coul != 0.0) {
            double qq = COULOMB_KCAL * a->charge[i] * a->charge[j];
            v += scale_coul * (qq / r);
            f_radial += scale_coul * (qq / r2);
        }
        potential += v;
        double gx = f_radial * dx / r, gy = f_radial * dy / r, gz = f_radial * dz / r;
        fx[i] -= gx; fy[i] -= gy; fz[i] -= gz;
        fx[j] += gx; fy[j] += gy; fz[j] += gz;
    }
    return potential;
}

double or_pair14_forces(const double *px, const double *py, const double *pz, const or_atoms *a,
                        const uint32_t *p14_i, const uint32_t *p14_j, int64_t n14,
                        double scale_lj, double scale_coul, int32_t coulomb,
                        double *fx, double *fy, double *fz) {
    return or_pair14_forces_box(px, py, pz, a, p14_i, p14_j, n14, scale_lj, scale_coul, coulomb, NULL, fx, fy, fz);
}

/* -------------------------------------------------------------- bonded */

double or_bond_forces_box(const double *px, const double *py, const double *pz, const or_topology *t,
                          const double *mi_box, double *fx, double *fy, double *fz) {
    /* force/bonded.rs:5-40 */
    double potential = 0.0;
    for (int64_t n = 0; n < t->n_bonds; n++) {
        uint32_t i = t->bond_i[n], j = t->bond_j[n];
        double k = t->bond_k[n], r0 = t->bond_r0[n];
        double dx = bdiff(px[j] - px[i], mi_box, 0);
        double dy = bdiff(py[j] - py[i], mi_box, 1);
        double dz = bdiff(pz[j] - pz[i], mi_box, 2);
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        if (r == 0.0) continue;
        double dv_dr = 2.0 * k * (r - r0);
        potential += k * (r - r0) * (r - r0);
        double ux = dx / r, uy = dy / r, uz = dz / r;
        fx[i] += dv_dr * ux; fy[i] += dv_dr * uy; fz[i] += dv_dr * uz;
        fx[j] -= dv_dr * ux; fy[j] -= dv_dr * uy; fz[j] -= dv_dr * uz;
    }
    return potential;
}

double or_bond_forces(const double *px, const double *py, const double *pz, const or_topology *t,
                      double *fx, double *fy, double *fz) {
    return or_bond_forces_box(px, py, pz, t, NULL, fx, fy, fz);
}

static double clamp_rs(double x, double lo, double hi) {
    /* Rust f64::clamp: NaN passes through */
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

double or_angle_forces_box(const double *px, const double *py, const double *pz, const or_topology *t,
                           const double *mi_box, double *fx, double *fy, double *fz) {
    /* force/bonded.rs:44-102 */
    double potential = 0.0;
    for (int64_t n = 0; n < t->n_angles; n++) {
        uint32_t i = t->angle_i[n], j = t->angle_j[n], kk = t->angle_k[n];
        double k_const = t->angle_kth[n], theta0 = t->angle_th0[n];
        double b1[3] = {bdiff(px[i] - px[j], mi_box, 0), bdiff(py[i] - py[j], mi_box, 1),
                        bdiff(pz[i] - pz[j], mi_box, 2)};
        double b2[3] = {bdiff(px[kk] - px[j], mi_box, 0), bdiff(py[kk] - py[j], mi_box, 1),
                        bdiff(pz[kk] - pz[j], mi_box, 2)};
        double r1 = sqrt(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
        double r2 = sqrt(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
        if (r1 == 0.0 || r2 == 0.0) continue;
        double dot = b1[0] * b2[0] + b1[1] * b2[1] + b1[2] * b2[2];
        double cos_theta = clamp_rs(dot / (r1 * r2), -1.0, 1.0);
        double sin_theta = fmax(sqrt(1.0 - cos_theta * cos_theta), 1e-8);
        double theta = acos(cos_theta);
        double dv_dtheta = 2.0 * k_const * (theta - theta0);
        potential += k_const * (theta - theta0) * (theta - theta0);
        double aa = dv_dtheta / sin_theta;
        double f_i[3], f_k[3];
        for (int c = 0; c < 3; c++) {
            f_i[c] = aa * (b2[c] / (r1 * r2) - cos_theta * b1[c] / (r1 * r1));
            f_k[c] = aa * (b1[c] / (r1 * r2) - cos_theta * b2[c] / (r2 * r2));
        }
        fx[i] += f_i[0]; fy[i] += f_i[1]; fz[i] += f_i[2];
        fx[kk] += f_k[0]; fy[kk] += f_k[1]; fz[kk] += f_k[2];
        fx[j] -= f_i[0] + f_k[0]; fy[j] -= f_i[1] + f_k[1]; fz[j] -= f_i[2] + f_k[2];
    }
    return potential;
}

double or_angle_forces(const double *px, const double *py, const double *pz, const or_topology *t,
                       double *fx, double *fy, double *fz) {
    return or_angle_forces_box(px, py, pz, t, NULL, fx, fy, fz);
}

static void v_sub(const double *a, const double *b, double *o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; }
static void v_add(const double *a, const double *b, double *o) { o[0] = a[0] + b[0]; o[1] = a[1] + b[1]; o[2] = a[2] + b[2]; }
static void v_cross(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static double v_dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void v_scale(const double *a, double s, double *o) { o[0] = a[0] * s; o[1] = a[1] * s; o[2] = a[2] * s; }

double or_dihedral_forces_box(const double *px, const double *py, const double *pz, const or_topology *t,
                              const double *mi_box, double *fx, double *fy, double *fz) {
    /* force/bonded.rs:112-164 */
    double potential = 0.0;
    for (int64_t n = 0; n < t->n_diheds; n++) {
        uint32_t i = t->dihed_i[n], j = t->dihed_j[n], k = t->dihed_k[n], l = t->dihed_l[n];
        double k_phi = t->dihed_kphi[n];
        double mult = (double)t->dihed_n[n];
        double delta = t->dihed_delta[n];
        double pi_[3] = {px[i], py[i], pz[i]}, pj[3] = {px[j], py[j], pz[j]};
        double pk[3] = {px[k], py[k], pz[k]}, pl[3] = {px[l], py[l], pz[l]};
        double b1[3], b2[3], b3[3], m[3], nv[3];
        v_sub(pj, pi_, b1);
        v_sub(pk, pj, b2);
        v_sub(pl, pk, b3);
        for (int c = 0; c < 3; c++) {
            b1[c] = bdiff(b1[c], mi_box, c);
            b2[c] = bdiff(b2[c], mi_box, c);
            b3[c] = bdiff(b3[c], mi_box, c);
        }
        v_cross(b1, b2, m);
        v_cross(b2, b3, nv);
        double m_len2 = v_dot(m, m);
        double n_len2 = v_dot(nv, nv);
        double b2_len = sqrt(v_dot(b2, b2));
        if (m_len2 == 0.0 || n_len2 == 0.0 || b2_len == 0.0) continue;
        double x = v_dot(m, nv);
        double mxn[3];
        v_cross(m, nv, mxn);
        double y = v_dot(mxn, b2) / b2_len;
        double phi = atan2(y, x);
        potential += k_phi * (1.0 + cos(mult * phi - delta));
        double dv_dphi = k_phi * mult * sin(mult * phi - delta);
        double f_i[3], f_l[3], f_j[3], f_k[3], t1[3], t2[3];
        v_scale(m, -dv_dphi * b2_len / m_len2, f_i);
        v_scale(nv, dv_dphi * b2_len / n_len2, f_l);
        double p = v_dot(b1, b2) / (b2_len * b2_len);
        double q = v_dot(b3, b2) / (b2_len * b2_len);
        v_scale(f_i, -(p + 1.0), t1);
        v_scale(f_l, q, t2);
        v_add(t1, t2, f_j);
        v_scale(f_i, p, t1);
        v_scale(f_l, q + 1.0, t2);
        v_sub(t1, t2, f_k);
        fx[i] += f_i[0]; fy[i] += f_i[1]; fz[i] += f_i[2];
        fx[j] += f_j[0]; fy[j] += f_j[1]; fz[j] += f_j[2];
        fx[k] += f_k[0]; fy[k] += f_k[1]; fz[k] += f_k[2];
        fx[l] += f_l[0]; fy[l] += f_l[1]; fz[l] += f_l[2];
    }
    return potential;
}

double or_dihedral_forces(const double *px, const double *py, const double *pz, const or_topology *t,
                          double *fx, double *fy, double *fz) {
    return or_dihedral_forces_box(px, py, pz, t, NULL, fx, fy, fz);
}

/* ---------------------------------------------------------- constraints */

int64_t or_constraint_solve_box(const or_topology *t, const or_atoms *a,
                                const double *rx, const double *ry, const double *rz,
                                double *px, double *py, double *pz,
                                uint32_t max_iter, double tol, uint64_t step,
                                const double *lam0, double *lam_out, const double *mi_box,
                                or_convergence_error *err) {
    /* constraint.rs:62-152 */
    int64_t n_constr = t->n_constr;
    if (n_constr == 0) return 0;
    int64_t n_atoms = a->n;
    double *dx_ = (double *)calloc((size_t)n_atoms * 3, sizeof(double));
    double *dy_ = dx_ + n_atoms, *dz_ = dy_ + n_atoms;
    if (lam_out) for (int64_t c = 0; c < n_constr; c++) lam_out[c] = lam0 ? lam0[c] : 0.0;
    if (lam0) {
        /* warm start: one displacement with the predicted multipliers, same
         * update formula as a Jacobi sweep (constraint.rs:116-121, 130-134) */
        for (int64_t c = 0; c < n_constr; c++) {
            uint32_t i = t->constr_i[c], j = t->constr_j[c];
            double rxx = bdiff(rx[i] - rx[j], mi_box, 0), ryy = bdiff(ry[i] - ry[j], mi_box, 1);
            double rzz = bdiff(rz[i] - rz[j], mi_box, 2);
            double inv_mi = 1.0 / a->mass[i], inv_mj = 1.0 / a->mass[j];
            double lambda = lam0[c];
            dx_[i] -= lambda * inv_mi * rxx; dy_[i] -= lambda * inv_mi * ryy; dz_[i] -= lambda * inv_mi * rzz;
            dx_[j] += lambda * inv_mj * rxx; dy_[j] += lambda * inv_mj * ryy; dz_[j] += lambda * inv_mj * rzz;
        }
        for (int64_t q = 0; q < n_atoms; q++) { px[q] += dx_[q]; py[q] += dy_[q]; pz[q] += dz_[q]; }
    }
    double last_max_lambda = 0.0;
    int64_t lw0 = 0, lw1 = 0, lw2 = 0;
    for (uint32_t iter = 0; iter < max_iter; iter++) {
        memset(dx_, 0, sizeof(double) * (size_t)n_atoms * 3);
        double max_lambda = 0.0;
        int64_t w0 = 0, w1 = 0, w2 = 0;
        for (int64_t c = 0; c < n_constr; c++) {
            uint32_t i = t->constr_i[c], j = t->constr_j[c];
            double dsq_target = t->constr_dsq[c];
            double dx = bdiff(px[i] - px[j], mi_box, 0);
            double dy = bdiff(py[i] - py[j], mi_box, 1);
            double dz = bdiff(pz[i] - pz[j], mi_box, 2);
            double diff = dx * dx + dy * dy + dz * dz - dsq_target;
            double rxx = bdiff(rx[i] - rx[j], mi_box, 0);
            double ryy = bdiff(ry[i] - ry[j], mi_box, 1);
            double rzz = bdiff(rz[i] - rz[j], mi_box, 2);
            double inv_mi = 1.0 / a->mass[i];
            double inv_mj = 1.0 / a->mass[j];
            double dot_new_old = dx * rxx + dy * ryy + dz * rzz;
            double denom = 2.0 * (inv_mi + inv_mj) * dot_new_old;
            double lambda = denom == 0.0 ? 0.0 : diff / denom;
            dx_[i] -= lambda * inv_mi * rxx; dy_[i] -= lambda * inv_mi * ryy; dz_[i] -= lambda * inv_mi * rzz;
            dx_[j] += lambda * inv_mj * rxx; dy_[j] += lambda * inv_mj * ryy; dz_[j] += lambda * inv_mj * rzz;
            if (lam_out) lam_out[c] += lambda;
            double la = fabs(lambda);
            if (la > max_lambda) { max_lambda = la; w0 = c; w1 = i; w2 = j; }
        }
        for (int64_t q = 0; q < n_atoms; q++) { px[q] += dx_[q]; py[q] += dy_[q]; pz[q] += dz_[q]; }
        if (max_lambda < tol) { free(dx_); return (int64_t)iter + 1; }
        last_max_lambda = max_lambda; lw0 = w0; lw1 = w1; lw2 = w2;
    }
    free(dx_);
    if (err) {
        err->step = step; err->constraint_idx = lw0; err->atom_i = lw1; err->atom_j = lw2;
        err->residual = last_max_lambda; err->max_iter = max_iter;
    }
    return -1;
}

int64_t or_constraint_solve_ws(const or_topology *t, const or_atoms *a,
                               const double *rx, const double *ry, const double *rz,
                               double *px, double *py, double *pz,
                               uint32_t max_iter, double tol, uint64_t step,
                               const double *lam0, double *lam_out, or_convergence_error *err) {
    return or_constraint_solve_box(t, a, rx, ry, rz, px, py, pz, max_iter, tol, step, lam0, lam_out, NULL, err);
}

int64_t or_constraint_solve(const or_topology *t, const or_atoms *a,
                            const double *rx, const double *ry, const double *rz,
                            double *px, double *py, double *pz,
                            uint32_t max_iter, double tol, uint64_t step, or_convergence_error *err) {
    return or_constraint_solve_box(t, a, rx, ry, rz, px, py, pz, max_iter, tol, step, NULL, NULL, NULL, err);
}

int64_t or_constrain_velocities_box(const or_topology *t, const or_atoms *a,
                                    const double *px, const double *py, const double *pz,
                                    double *vx, double *vy, double *vz,
                                    uint32_t max_iter, double tol, uint64_t step, const double *mi_box,
                                    or_convergence_error *err) {
    /* constraint.rs:170-259 */
    int64_t n_constr = t->n_constr;
    if (n_constr == 0) return 0;
    int64_t n_atoms = a->n;
    double *dx_ = (double *)calloc((size_t)n_atoms * 3, sizeof(double));
    double *dy_ = dx_ + n_atoms, *dz_ = dy_ + n_atoms;
    double last_max_mu = 0.0;
    int64_t lw0 = 0, lw1 = 0, lw2 = 0;
    for (uint32_t iter = 0; iter < max_iter; iter++) {
        memset(dx_, 0, sizeof(double) * (size_t)n_atoms * 3);
        double max_mu = 0.0;
        int64_t w0 = 0, w1 = 0, w2 = 0;
        for (int64_t c = 0; c < n_constr; c++) {
            uint32_t i = t->constr_i[c], j = t->constr_j[c];
            double rxx = bdiff(px[i] - px[j], mi_box, 0);
            double ryy = bdiff(py[i] - py[j], mi_box, 1);
            double rzz = bdiff(pz[i] - pz[j], mi_box, 2);
            double rsq = rxx * rxx + ryy * ryy + rzz * rzz;
            double dvx = vx[i] - vx[j];
            double dvy = vy[i] - vy[j];
            double dvz = vz[i] - vz[j];
            double rel_vel = dvx * rxx + dvy * ryy + dvz * rzz;
            double inv_mi = 1.0 / a->mass[i];
            double inv_mj = 1.0 / a->mass[j];
            double denom = (inv_mi + inv_mj) * rsq;
            double mu = denom == 0.0 ? 0.0 : rel_vel / denom;
            dx_[i] -= mu * inv_mi * rxx; dy_[i] -= mu * inv_mi * ryy; dz_[i] -= mu * inv_mi * rzz;
            dx_[j] += mu * inv_mj * rxx; dy_[j] += mu * inv_mj * ryy; dz_[j] += mu * inv_mj * rzz;
            double ma = fabs(mu);
            if (ma > max_mu) { max_mu = ma; w0 = c; w1 = i; w2 = j; }
        }
        for (int64_t q = 0; q < n_atoms; q++) { vx[q] += dx_[q]; vy[q] += dy_[q]; vz[q] += dz_[q]; }
        if (max_mu < tol) { free(dx_); return (int64_t)iter + 1; }
        last_max_mu = max_mu; lw0 = w0; lw1 = w1; lw2 = w2;
    }
    free(dx_);
    if (err) {
        err->step = step; err->constraint_idx = lw0; err->atom_i = lw1; err->atom_j = lw2;
        err->residual = last_max_mu; err->max_iter = max_iter;
    }
    return -1;
}

int64_t or_constrain_velocities(const or_topology *t, const or_atoms *a,
                                const double *px, const double *py, const double *pz,
                                double *vx, double *vy, double *vz,
                                uint32_t max_iter, double tol, uint64_t step, or_convergence_error *err) {
    return or_constrain_velocities_box(t, a, px, py, pz, vx, vy, vz, max_iter, tol, step, NULL, err);
}

/* ---------------------------------------------------------- integrator */

#define FORCE_TO_ACCEL_ANG_PER_PS2 (20.455 * 20.455) /* integrator.rs:9 */

void or_half_kick(int64_t n, double *vx, double *vy, double *vz,
                  const double *fx, const double *fy, const double *fz, const double *mass, double dt_half) {
    /* integrator.rs:14-21 */
    for (int64_t i = 0; i < n; i++) {
        double inv_m = 1.0 / mass[i];
        vx[i] += dt_half * fx[i] * inv_m * FORCE_TO_ACCEL_ANG_PER_PS2;
        vy[i] += dt_half * fy[i] * inv_m * FORCE_TO_ACCEL_ANG_PER_PS2;
        vz[i] += dt_half * fz[i] * inv_m * FORCE_TO_ACCEL_ANG_PER_PS2;
    }
}

int64_t or_drift_and_constrain_box(int64_t n, double *px, double *py, double *pz,
                                   double *vx, double *vy, double *vz, const or_topology *t, const or_atoms *a,
                                   double dt, uint32_t max_iter, double tol, uint64_t step, const double *mi_box,
                                   or_convergence_error *err) {
    /* integrator.rs:32-71 */
    double *ref = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * 3);
    double *rx = ref, *ry = ref + n, *rz = ref + 2 * n;
    memcpy(rx, px, sizeof(double) * (size_t)n);
    memcpy(ry, py, sizeof(double) * (size_t)n);
    memcpy(rz, pz, sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        px[i] += dt * vx[i];
        py[i] += dt * vy[i];
        pz[i] += dt * vz[i];
    }
    int64_t iters = or_constraint_solve_box(t, a, rx, ry, rz, px, py, pz, max_iter, tol, step, NULL, NULL, mi_box,
                                            err);
    if (iters < 0) { free(ref); return iters; }
    for (int64_t i = 0; i < n; i++) {
        vx[i] = (px[i] - rx[i]) / dt;
        vy[i] = (py[i] - ry[i]) / dt;
        vz[i] = (pz[i] - rz[i]) / dt;
    }
    free(ref);
    return iters;
}

int64_t or_drift_and_constrain(int64_t n, double *px, double *py, double *pz,
                               double *vx, double *vy, double *vz, const or_topology *t, const or_atoms *a,
                               double dt, uint32_t max_iter, double tol, uint64_t step,
                               or_convergence_error *err) {
    return or_drift_and_constrain_box(n, px, py, pz, vx, vy, vz, t, a, dt, max_iter, tol, step, NULL, err);
}

double or_kinetic_energy(int64_t n, const double *vx, const double *vy, const double *vz, const double *mass) {
    /* geodesic/src/lib.rs:25,68-77 */
    double sum = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        sum += mass[i] * v2;
    }
    return 0.5 * sum * (1.0 / (20.455 * 20.455));
}

/* ---------------------------------------------------------- CpuBackend */

struct or_backend {
    or_atoms atoms;
    or_topology topo;
    or_params params;
    int32_t n_threads;
    int64_t n_pairs, cap;
    uint32_t *pair_i, *pair_j;
    double *ref;           /* ref_x | ref_y | ref_z */
    double *thread_buf;    /* T x 3N */
    double *thread_energy; /* T */
    double *bonded_buf;    /* 3N */
    uint32_t *p14_i, *p14_j;
    int64_t n14;
};

int32_t or_host_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int32_t)n : 1;
}

or_backend *or_backend_new(const or_atoms *a, const or_topology *t, const or_params *p) {
    /* cpu_backend.rs:50-83 */
    or_backend *b = (or_backend *)calloc(1, sizeof(or_backend));
    b->atoms = *a;
    b->topo = *t;
    b->params = *p;
    int32_t nt = p->n_threads == 0 ? or_host_threads() : p->n_threads;
    b->n_threads = nt < 1 ? 1 : nt;
    int64_t n = a->n;
    b->ref = (double *)calloc((size_t)(n > 0 ? n : 1) * 3, sizeof(double));
    b->thread_buf = (double *)calloc((size_t)b->n_threads * (size_t)(n > 0 ? n : 1) * 3, sizeof(double));
    b->thread_energy = (double *)calloc((size_t)b->n_threads, sizeof(double));
    b->bonded_buf = (double *)calloc((size_t)(n > 0 ? n : 1) * 3, sizeof(double));
    if (p->scale14_lj != 0.0 || (p->coulomb && p->scale14_coul != 0.0)) {
        int64_t cnt = or_pairs14(t, n, 0, NULL, NULL);
        b->p14_i = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(cnt > 0 ? cnt : 1));
        b->p14_j = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(cnt > 0 ? cnt : 1));
        b->n14 = or_pairs14(t, n, cnt, b->p14_i, b->p14_j);
    }
    return b;
}

void or_backend_free(or_backend *b) {
    if (!b) return;
    free(b->pair_i); free(b->pair_j); free(b->ref); free(b->thread_buf); free(b->thread_energy);
    free(b->bonded_buf); free(b->p14_i); free(b->p14_j); free(b);
}

int32_t or_backend_n_threads(const or_backend *b) { return b->n_threads; }

int64_t or_backend_build_neighbor_list(or_backend *b, double *px, double *py, double *pz) {
    /* cpu_backend.rs:88-90 -> neighbor::build */
    int64_t n = b->atoms.n;
    int64_t cnt = or_neighbor_build(n, px, py, pz, &b->params, &b->topo, b->cap, b->pair_i, b->pair_j);
    for (;;) {
        if (cnt <= b->cap) { b->n_pairs = cnt; break; }
        free(b->pair_i); free(b->pair_j);
        b->cap = cnt + cnt / 8 + 16;
        b->pair_i = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)b->cap);
        b->pair_j = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)b->cap);
        /* the positions are wrapped already: fetch the pairs only */
        cnt = or_neighbor_pairs(n, px, py, pz, &b->params, &b->topo, b->cap, b->pair_i, b->pair_j, 0);
    }
    memcpy(b->ref, px, sizeof(double) * (size_t)n);
    memcpy(b->ref + n, py, sizeof(double) * (size_t)n);
    memcpy(b->ref + 2 * n, pz, sizeof(double) * (size_t)n);
    return b->n_pairs;
}

int64_t or_backend_set_pairs(or_backend *b, int64_t n_pairs, const uint32_t *pair_i, const uint32_t *pair_j,
                             const double *px, const double *py, const double *pz) {
    int64_t n = b->atoms.n;
    if (n_pairs > b->cap) {
        free(b->pair_i); free(b->pair_j);
        b->cap = n_pairs;
        b->pair_i = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n_pairs > 0 ? n_pairs : 1));
        b->pair_j = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n_pairs > 0 ? n_pairs : 1));
    }
    memcpy(b->pair_i, pair_i, sizeof(uint32_t) * (size_t)n_pairs);
    memcpy(b->pair_j, pair_j, sizeof(uint32_t) * (size_t)n_pairs);
    b->n_pairs = n_pairs;
    memcpy(b->ref, px, sizeof(double) * (size_t)n);
    memcpy(b->ref + n, py, sizeof(double) * (size_t)n);
    memcpy(b->ref + 2 * n, pz, sizeof(double) * (size_t)n);
    return n_pairs;
}

int64_t or_backend_pairs(const or_backend *b, const uint32_t **pair_i, const uint32_t **pair_j) {
    *pair_i = b->pair_i;
    *pair_j = b->pair_j;
    return b->n_pairs;
}

typedef struct {
    or_backend *b;
    const double *px, *py, *pz;
    int k;
    int64_t chunk;
} strip_job;

static void *strip_worker(void *arg) {
    /* cpu_backend.rs:141-161: thread k owns the contiguous strip
     * [k*chunk, (k+1)*chunk) of the flat pair list and a private buffer */
    strip_job *j = (strip_job *)arg;
    or_backend *b = j->b;
    int64_t n = b->atoms.n;
    double *buf = b->thread_buf + (size_t)j->k * (size_t)n * 3;
    memset(buf, 0, sizeof(double) * (size_t)n * 3);
    int64_t start = j->k * j->chunk, end = (j->k + 1) * j->chunk;
    if (start > b->n_pairs) start = b->n_pairs;
    if (end > b->n_pairs) end = b->n_pairs;
    double e = 0.0;
    if (start < end) {
        e = or_pair_forces(j->px, j->py, j->pz, &b->atoms, b->pair_i + start, b->pair_j + start, end - start,
                           b->params.r_cutoff, b->params.r_switch, b->params.box, buf, buf + n, buf + 2 * n);
        if (b->params.coulomb)
            e += or_coulomb_forces(j->px, j->py, j->pz, &b->atoms, b->pair_i + start, b->pair_j + start,
                                   end - start, b->params.r_cutoff, b->params.r_switch, b->params.box,
                                   buf, buf + n, buf + 2 * n);
    }
    b->thread_energy[j->k] = e;
    return NULL;
}

double or_backend_compute_forces(or_backend *b, const double *px, const double *py, const double *pz,
                                 double *fx, double *fy, double *fz) {
    /* cpu_backend.rs:92-182 */
    int64_t n = b->atoms.n;
    double *bf = b->bonded_buf;
    memset(bf, 0, sizeof(double) * (size_t)n * 3);
    double potential = 0.0;
    const double *mb = mi_box_of(&b->params);
    potential += or_bond_forces_box(px, py, pz, &b->topo, mb, bf, bf + n, bf + 2 * n);
    potential += or_angle_forces_box(px, py, pz, &b->topo, mb, bf, bf + n, bf + 2 * n);
    potential += or_dihedral_forces_box(px, py, pz, &b->topo, mb, bf, bf + n, bf + 2 * n);
    if (b->n14)
        potential += or_pair14_forces_box(px, py, pz, &b->atoms, b->p14_i, b->p14_j, b->n14, b->params.scale14_lj,
                                          b->params.scale14_coul, b->params.coulomb, mb, bf, bf + n, bf + 2 * n);
    int nt = b->n_threads;
    int64_t chunk = (b->n_pairs + nt - 1) / nt;
    if (chunk < 1) chunk = 1;
    strip_job *jobs = (strip_job *)malloc(sizeof(strip_job) * (size_t)nt);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
    for (int k = 0; k < nt; k++) {
        jobs[k] = (strip_job){b, px, py, pz, k, chunk};
        if (k > 0) pthread_create(&th[k], NULL, strip_worker, &jobs[k]);
    }
    strip_worker(&jobs[0]);
    for (int k = 1; k < nt; k++) pthread_join(th[k], NULL);
    free(th); free(jobs);
    /* cpu_backend.rs:164-166: energy in thread-index order */
    for (int k = 0; k < nt; k++) potential += b->thread_energy[k];
    /* cpu_backend.rs:170-179: bonded, then threads 0..T-1 */
    memcpy(fx, bf, sizeof(double) * (size_t)n);
    memcpy(fy, bf + n, sizeof(double) * (size_t)n);
    memcpy(fz, bf + 2 * n, sizeof(double) * (size_t)n);
    for (int k = 0; k < nt; k++) {
        const double *buf = b->thread_buf + (size_t)k * (size_t)n * 3;
        for (int64_t i = 0; i < n; i++) {
            fx[i] += buf[i];
            fy[i] += buf[n + i];
            fz[i] += buf[2 * n + i];
        }
    }
    return potential;
}

int32_t or_backend_needs_rebuild(const or_backend *b, const double *px, const double *py, const double *pz) {
    int64_t n = b->atoms.n;
    return or_needs_rebuild(n, px, py, pz, b->ref, b->ref + n, b->ref + 2 * n, b->params.r_skin, b->params.r_cutoff);
}

int64_t or_backend_geodesic_drift(or_backend *b, double *px, double *py, double *pz,
                                  double *vx, double *vy, double *vz, double dt, uint64_t step,
                                  or_convergence_error *err) {
    /* cpu_backend.rs:184-194 */
    return or_drift_and_constrain_box(b->atoms.n, px, py, pz, vx, vy, vz, &b->topo, &b->atoms, dt,
                                      b->params.max_constr_iter, b->params.constr_tol, step, mi_box_of(&b->params),
                                      err);
}

/* ------------------------------------------------------------- run loop */

static int all_finite(int64_t n, const double *x, const double *y, const double *z) {
    for (int64_t i = 0; i < n; i++)
        if (!isfinite(x[i]) || !isfinite(y[i]) || !isfinite(z[i])) return 0;
    return 1;
}

int64_t or_run(const or_atoms *a, const or_topology *t, const or_params *p,
               double *px, double *py, double *pz, double *vx, double *vy, double *vz,
               double dt, uint64_t n_steps, uint32_t frame_interval, int64_t max_frames,
               float *frames, double *pot, double *kin, uint64_t *fail_step, or_convergence_error *err) {
    /* geodesic/src/lib.rs:187-333 */
    int64_t n = a->n;
    or_backend *b = or_backend_new(a, t, p);
    double *f = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * 3);
    double *fx = f, *fy = f + n, *fz = f + 2 * n;
    int64_t n_frames = 0, rc = 0;
    uint64_t step = 0;
    or_backend_build_neighbor_list(b, px, py, pz);
    double pe = or_backend_compute_forces(b, px, py, pz, fx, fy, fz);
    if (!all_finite(n, fx, fy, fz)) { rc = -2; goto done; }
    if (or_constrain_velocities_box(&b->topo, a, px, py, pz, vx, vy, vz, p->max_constr_iter, p->constr_tol, 0,
                                    mi_box_of(p), err) < 0) {
        rc = -1; goto done;
    }
#define EMIT_FRAME()                                                                  \
    do {                                                                              \
        if (n_frames < max_frames) {                                                  \
            float *fr = frames + (size_t)n_frames * 3 * (size_t)n;                    \
            for (int64_t i = 0; i < n; i++) {                                         \
                fr[i] = (float)px[i]; fr[n + i] = (float)py[i]; fr[2 * n + i] = (float)pz[i]; \
            }                                                                         \
            pot[n_frames] = pe;                                                       \
            kin[n_frames] = or_kinetic_energy(n, vx, vy, vz, a->mass);                \
        }                                                                             \
        n_frames++;                                                                   \
    } while (0)
    EMIT_FRAME();
    for (uint64_t s = 0; s < n_steps; s++) {
        or_half_kick(n, vx, vy, vz, fx, fy, fz, a->mass, dt / 2.0);
        if (or_backend_geodesic_drift(b, px, py, pz, vx, vy, vz, dt, step, err) < 0) { rc = -1; goto done; }
        if (!all_finite(n, px, py, pz)) { rc = -3; goto done; }
        if (or_backend_needs_rebuild(b, px, py, pz)) or_backend_build_neighbor_list(b, px, py, pz);
        pe = or_backend_compute_forces(b, px, py, pz, fx, fy, fz);
        if (!all_finite(n, fx, fy, fz)) { rc = -2; goto done; }
        or_half_kick(n, vx, vy, vz, fx, fy, fz, a->mass, dt / 2.0);
        if (or_constrain_velocities_box(&b->topo, a, px, py, pz, vx, vy, vz, p->max_constr_iter, p->constr_tol,
                                        step, mi_box_of(p), err) < 0) {
            rc = -1; goto done;
        }
        step += 1;
        if (step % frame_interval == 0) EMIT_FRAME();
    }
#undef EMIT_FRAME
    rc = n_frames;
done:
    if (fail_step) *fail_step = step;
    free(f);
    or_backend_free(b);
    return rc;
}
